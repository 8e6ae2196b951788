// Shared-memory FFTs for power-of-two lengths 2..256, used by the fused
// spectral passes (hpf_spectral.cu).
//
// A batch of 1-D transforms over float2 data in shared memory is done in two
// steps (the four-step method, N = N1 * N2): N2 transforms of length N1 over
// the elements n = N2*n1 + n2 in registers, a twiddle w_N^(n2 k1), then N1
// transforms of length N2 over contiguous runs, again in registers.  The
// result is left in place in digit-transposed order: frequency k = k1 + N1*k2
// sits at element N2*k1 + k2 (FftIdx::pos below), so no reordering pass or
// extra buffer is needed; the callers read through the index maps.
//
// Sign convention as cuFFT / FFTW: forward exp(-2 pi i k n / N), inverse
// exp(+2 pi i k n / N), both unnormalised.  The in-register radix-2 stages use
// the exact values of cos and sin at multiples of 2 pi / 16; the twiddles of
// the middle step come from a table exp(-2 pi i m / 512) computed on the host
// in double precision.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hpf_fft {

constexpr int kTableN = 512;  // twiddle table length: exp(-2 pi i m / 512)

// (loops, not recursion, so that they fold to constants once the callers'
// loops are unrolled)
__host__ __device__ constexpr int ilog2(int n) {
    int b = 0;
    while ((1 << b) < n) ++b;
    return b;
}
__host__ __device__ __forceinline__ constexpr int bitrev(int i, int bits) {
    int r = 0;
    for (int b = 0; b < bits; ++b) r |= ((i >> b) & 1) << (bits - 1 - b);
    return r;
}
// first-step length N1 of the split N = N1 * N2 (N1 <= 16, N2 <= 16; N1 = 8
// from 32 to 128 keeps the per-thread arrays of the first step short)
__host__ __device__ constexpr int split1(int n) {
    return n <= 16 ? n : (n <= 128 ? 8 : 16);
}

__device__ __forceinline__ float2 c_add(float2 a, float2 b) {
    return make_float2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) {
    return make_float2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ float2 c_mul(float2 a, float2 w) {
    return make_float2(fmaf(a.x, w.x, -a.y * w.y), fmaf(a.x, w.y, a.y * w.x));
}
__device__ __forceinline__ float2 c_conj(float2 a) { return make_float2(a.x, -a.y); }

// v * exp(-+2 pi i m / 16) for m = 0..7 (compile-time after unrolling); the
// products by 1 and by -+i are exact sign and swap operations.
template <bool INV>
__device__ __forceinline__ float2 rot16(float2 v, int m) {
    constexpr float c1 = 0.92387953251128675613f;  // cos(pi/8)
    constexpr float c2 = 0.70710678118654752440f;  // cos(pi/4)
    constexpr float c3 = 0.38268343236508977173f;  // cos(3pi/8)
    if (m == 0) return v;
    if (m == 4) return INV ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
    float cr, si;  // cos(2 pi m/16), sin(2 pi m/16)
    switch (m) {
        case 1: cr = c1; si = c3; break;
        case 2: cr = c2; si = c2; break;
        case 3: cr = c3; si = c1; break;
        case 5: cr = -c3; si = c1; break;
        case 6: cr = -c2; si = c2; break;
        default: cr = -c1; si = c3; break;  // m == 7
    }
    return c_mul(v, make_float2(cr, INV ? si : -si));
}

// In-register radix-2 transform of length R <= 16, natural order in and out.
template <int R, bool INV>
__device__ __forceinline__ void reg_fft(float2 (&a)[R]) {
    static_assert(R >= 1 && R <= 16 && (R & (R - 1)) == 0, "register FFT length");
    constexpr int bits = ilog2(R);
    float2 b[R];
#pragma unroll
    for (int i = 0; i < R; ++i) b[bitrev(i, bits)] = a[i];
#pragma unroll
    for (int h = 1; h < R; h <<= 1) {
#pragma unroll
        for (int i0 = 0; i0 < R; i0 += 2 * h) {
#pragma unroll
            for (int j = 0; j < h; ++j) {
                const float2 u = b[i0 + j];
                const float2 v = rot16<INV>(b[i0 + j + h], j * (8 / h));
                b[i0 + j] = c_add(u, v);
                b[i0 + j + h] = c_sub(u, v);
            }
        }
    }
#pragma unroll
    for (int i = 0; i < R; ++i) a[i] = b[i];
}

// Index maps of a length-n transform's digit-transposed order, as shifts
// and masks (n a power of two <= 256): pos(k) is the element holding
// frequency k, freq(p) the frequency held by element p.
struct FftIdx {
    int n1s, n1m, n2s, n2m;
    __device__ __forceinline__ int pos(int k) const { return ((k & n1m) << n2s) + (k >> n1s); }
    __device__ __forceinline__ int freq(int p) const { return (p >> n2s) + ((p & n2m) << n1s); }
};
__device__ __forceinline__ FftIdx fft_idx(int n) {
    const int s = 31 - __clz(n);
    const int s1 = n <= 16 ? s : (n <= 128 ? 3 : 4);
    FftIdx f;
    f.n1s = s1;
    f.n1m = (1 << s1) - 1;
    f.n2s = s - s1;
    f.n2m = (1 << (s - s1)) - 1;
    return f;
}

// n / d for 0 <= n < 2^22 and a block-invariant d >= 1 (inv = 1.0f / d):
// the float quotient is within one of the truth, one correction step.
__device__ __forceinline__ int div_inv(int n, int d, float inv) {
    int q = __float2int_rz((float)n * inv);
    const int r = n - q * d;
    if (r >= d) ++q;
    else if (r < 0) --q;
    return q;
}

// Layout of a batch of transforms in shared memory: transform c (of count)
// starts at (c >> inner_shift) * s_outer + (c & inner_mask) * s_inner and
// its elements are es apart.
struct Batch {
    int count, inner_shift, s_outer, s_inner, es;
    float inv_count;
    __device__ __forceinline__ int base(int c) const {
        return (c >> inner_shift) * s_outer + (c & ((1 << inner_shift) - 1)) * s_inner;
    }
};
__device__ __forceinline__ Batch make_batch(int count, int inner_shift, int s_outer, int s_inner,
                                            int es) {
    Batch b;
    b.count = count;
    b.inner_shift = inner_shift;
    b.s_outer = s_outer;
    b.s_inner = s_inner;
    b.es = es;
    b.inv_count = 1.0f / (float)count;
    return b;
}

// Two-step transforms with caller-supplied element access, so that the
// first step can read from global memory (or compute its inputs) and the
// last can write to global memory, and shared memory is touched only
// between the steps.
//
// Step 1, item (c, n2): a[i] = ld(c, N2*i + n2) (natural element index),
// length-N1 transform in registers, twiddle, then st(c, N2*k1 + n2, a[k1])
// (the element position after step 1).  For N <= 16 (N2 = 1) step 1 is the
// whole transform and stores through fin(c, k, k, v) (natural index and
// position coincide).
// Step 2, item (c, k1): a[i] = ld(c, N2*k1 + i), length-N2 transform, then
// fin(c, k1 + N1*k2, N2*k1 + k2, a[k2]): the natural frequency and the
// position it came from.
// CFAST: neighbouring threads take neighbouring transforms c (for layouts
// where c is the unit stride); else neighbouring elements of one transform.
template <int V>
struct IntC {
    static constexpr int value = V;
};

struct NoPre {
    template <int R>
    __device__ __forceinline__ void operator()(int, int, float2 (&)[R]) const {}
};

// pre(c, n2, a): applied to an item's N1 loaded values (natural elements
// N2*i + n2) before its transform; the loads come first, all of them, so
// that they are in flight together.
template <int N, bool INV, bool CFAST, class LD, class ST, class FIN, class PRE = NoPre>
__device__ __forceinline__ void fft_step1(int count, float inv_count, LD ld, ST st, FIN fin,
                                          const float2* __restrict__ tw, PRE pre = PRE()) {
    constexpr int N1 = split1(N), N2 = N / N1;
    constexpr int TW = kTableN / N;
    const int items = count * N2;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        int c, n2;
        if (CFAST) {
            n2 = N2 == 1 ? 0 : div_inv(it, count, inv_count);
            c = it - n2 * count;
        } else {
            c = it / N2;
            n2 = it - c * N2;
        }
        float2 a[N1];
#pragma unroll
        for (int i = 0; i < N1; ++i) a[i] = ld(c, N2 * i + n2);
        pre(c, n2, a);
        reg_fft<N1, INV>(a);
        if (N2 == 1) {
#pragma unroll
            for (int k = 0; k < N1; ++k) fin(c, k, k, a[k]);
        } else {
#pragma unroll
            for (int k1 = 1; k1 < N1; ++k1) {
                float2 w = __ldg(tw + n2 * k1 * TW);
                if (INV) w.y = -w.y;
                a[k1] = c_mul(a[k1], w);
            }
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) st(c, N2 * k1 + n2, a[k1]);
        }
    }
}

template <int N, bool INV, bool CFAST, class LD, class FIN>
__device__ __forceinline__ void fft_step2(int count, float inv_count, LD ld, FIN fin) {
    constexpr int N1 = split1(N), N2 = N / N1;
    if (N2 == 1) return;
    const int items = count * N1;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        int c, k1;
        if (CFAST) {
            k1 = div_inv(it, count, inv_count);
            c = it - k1 * count;
        } else {
            c = it / N1;
            k1 = it - c * N1;
        }
        float2 a[N2];
#pragma unroll
        for (int i = 0; i < N2; ++i) a[i] = ld(c, N2 * k1 + i);
        reg_fft<N2, INV>(a);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) fin(c, k1 + N1 * k2, N2 * k1 + k2, a[k2]);
    }
}

// Calls f(IntC<n>()) for a runtime power of two n in [4, 256].
template <class F>
__device__ __forceinline__ void with_len(int n, F f) {
    switch (n) {
        case 4: f(IntC<4>()); break;
        case 8: f(IntC<8>()); break;
        case 16: f(IntC<16>()); break;
        case 32: f(IntC<32>()); break;
        case 64: f(IntC<64>()); break;
        case 128: f(IntC<128>()); break;
        default: f(IntC<256>()); break;
    }
}

// One batch of length-N transforms in shared memory, in place.  Transform c
// starts at L.base(c), its elements L.es apart; the result is left at the
// step-1 positions (FftIdx order).  All threads call it; the caller
// synchronises before and after.
template <int N, bool INV>
__device__ __forceinline__ void smem_fft(float2* buf, const Batch& L, const float2* __restrict__ tw) {
    auto at = [&](int c, int e) -> float2& { return buf[L.base(c) + e * L.es]; };
    auto ld = [&](int c, int e) { return at(c, e); };
    auto st = [&](int c, int p, float2 v) { at(c, p) = v; };
    auto fin = [&](int c, int k, int p, float2 v) { at(c, p) = v; };
    if (L.es == 1) {
        fft_step1<N, INV, false>(L.count, L.inv_count, ld, st, fin, tw);
        __syncthreads();
        fft_step2<N, INV, true>(L.count, L.inv_count, ld, fin);
    } else {
        fft_step1<N, INV, true>(L.count, L.inv_count, ld, st, fin, tw);
        __syncthreads();
        fft_step2<N, INV, true>(L.count, L.inv_count, ld, fin);
    }
}

template <bool INV>
__device__ __forceinline__ void smem_fft_n(int n, float2* buf, const Batch& L,
                                           const float2* __restrict__ tw) {
    with_len(n, [&](auto nc) { smem_fft<decltype(nc)::value, INV>(buf, L, tw); });
}

// ---- bulk copies global -> shared (TMA, completion on an mbarrier) -------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// dst, src 16-byte aligned; bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
        "[%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}
// Bounded wait for phase `parity` (a bulk copy that never lands would
// otherwise hang the block): false after ~2^22 polls (each try_wait itself
// suspends for a while), with the caller then recording an error.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (int i = 0; i < (1 << 22); ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

}  // namespace hpf_fft

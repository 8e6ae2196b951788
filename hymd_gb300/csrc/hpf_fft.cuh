// Shared-memory FFTs for lengths 2^a and 3 * 2^a up to 256, used by the
// fused spectral passes (hpf_spectral.cu).
//
// A batch of 1-D transforms is done in two steps (the four-step method,
// N = N1 * N2): N2 transforms of length N1 over the elements n = N2*n1 + n2
// in registers, a twiddle w_N^(n2 k1), then N1 transforms of length N2 over
// contiguous runs, again in registers.  The result is left in
// digit-transposed order: frequency k = k1 + N1*k2 sits at element N2*k1 + k2
// (Idx<N>::pos below), so no reordering pass or extra buffer is needed; the
// callers read through the index maps.
//
// Sign convention as cuFFT / FFTW: forward exp(-2 pi i k n / N), inverse
// exp(+2 pi i k n / N), both unnormalised.  The in-register transforms are
// radix 2 with the exact cos and sin of multiples of 2 pi / 16, and for
// lengths 3, 6, 12 one radix-3 stage (cos and sin of multiples of 2 pi / 12).
// The twiddles of the middle step come from tables exp(-2 pi i m / 512) and
// exp(-2 pi i m / 768) computed on the host in double precision.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hpf_fft {

// twiddle tables, back to back: exp(-2 pi i m / 512), m < 512, then
// exp(-2 pi i m / 768), m < 768
constexpr int kTable2 = 512;
constexpr int kTable3 = 768;
constexpr int kTableTotal = kTable2 + kTable3;

__host__ __device__ constexpr bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
// 2^a or 3 * 2^a
__host__ __device__ constexpr bool fft_len_ok(int n) {
    return is_pow2(n) || (n % 3 == 0 && is_pow2(n / 3));
}

// Twiddle m of length N: tw[Tw<N>::off + m * Tw<N>::stride].
template <int N>
struct Tw {
    static constexpr int off = is_pow2(N) ? 0 : kTable2;
    static constexpr int stride = (is_pow2(N) ? kTable2 : kTable3) / N;
};

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
// first-step length N1 of the split N = N1 * N2.  Powers of two: N1 = 8
// from 32 to 128, which keeps the per-thread arrays of the first step short.
// 3 * 2^a above 16: N1 the power of two (8 or 16), N2 = 3, 6 or 12.
__host__ __device__ constexpr int split1(int n) {
    return n <= 16 ? n
                   : (is_pow2(n) ? (n <= 128 ? 8 : 16) : (n % 16 == 0 ? 16 : 8));
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

// v * exp(-+2 pi i m / 12) for m = 0..11 (compile-time after unrolling).
template <bool INV>
__device__ __forceinline__ float2 rot12(float2 v, int m) {
    constexpr float s3 = 0.86602540378443864676f;  // sqrt(3)/2
    switch (m) {
        case 0: return v;
        case 3: return INV ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
        case 6: return make_float2(-v.x, -v.y);
        case 9: return INV ? make_float2(v.y, -v.x) : make_float2(-v.y, v.x);
        default: break;
    }
    float cr, si;  // cos(2 pi m/12), sin(2 pi m/12)
    switch (m) {
        case 1: cr = s3; si = 0.5f; break;
        case 2: cr = 0.5f; si = s3; break;
        case 4: cr = -0.5f; si = s3; break;
        case 5: cr = -s3; si = 0.5f; break;
        case 7: cr = -s3; si = -0.5f; break;
        case 8: cr = -0.5f; si = -s3; break;
        case 10: cr = 0.5f; si = -s3; break;
        default: cr = s3; si = -0.5f; break;  // m == 11
    }
    return c_mul(v, make_float2(cr, INV ? si : -si));
}

// Length-3 transform in place.
template <bool INV>
__device__ __forceinline__ void dft3(float2& b0, float2& b1, float2& b2) {
    constexpr float s3 = 0.86602540378443864676f;
    const float2 s = c_add(b1, b2), d = c_sub(b1, b2);
    const float2 t = make_float2(fmaf(-0.5f, s.x, b0.x), fmaf(-0.5f, s.y, b0.y));
    // -+i (sqrt(3)/2) d
    const float2 m = INV ? make_float2(-s3 * d.y, s3 * d.x) : make_float2(s3 * d.y, -s3 * d.x);
    b0 = c_add(b0, s);
    b1 = c_add(t, m);
    b2 = c_sub(t, m);
}

// In-register radix-2 transform of length R = 2^a <= 16, natural order in
// and out.
template <int R, bool INV>
__device__ __forceinline__ void reg_fft2(float2 (&a)[R]) {
    static_assert(R >= 1 && R <= 16 && is_pow2(R), "register FFT length");
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

// In-register transform of length R in {1, 2, 4, 8, 16, 3, 6, 12}: for
// R = 3P, a length-3 transform over n1 of x[P n1 + n2] for each n2, the
// twiddle w_R^(n2 k1), then length-P transforms over n2: X[k1 + 3 k2].
template <int R, bool INV>
__device__ __forceinline__ void reg_fft(float2 (&a)[R]) {
    if constexpr (R % 3 != 0) {
        reg_fft2<R, INV>(a);
    } else {
        constexpr int P = R / 3;
        static_assert(P == 1 || P == 2 || P == 4, "register FFT length");
        float2 y[3][P];
#pragma unroll
        for (int n2 = 0; n2 < P; ++n2) {
            float2 b0 = a[n2], b1 = a[P + n2], b2 = a[2 * P + n2];
            dft3<INV>(b0, b1, b2);
            y[0][n2] = b0;
            y[1][n2] = rot12<INV>(b1, (n2 * (12 / R)) % 12);
            y[2][n2] = rot12<INV>(b2, (2 * n2 * (12 / R)) % 12);
        }
#pragma unroll
        for (int k1 = 0; k1 < 3; ++k1) {
            reg_fft2<P, INV>(y[k1]);
#pragma unroll
            for (int k2 = 0; k2 < P; ++k2) a[k1 + 3 * k2] = y[k1][k2];
        }
    }
}

// Index maps of a length-N transform's digit-transposed order: pos(k) is
// the element holding frequency k, freq(p) the frequency held by element p.
template <int N>
struct Idx {
    static constexpr int N1 = split1(N), N2 = N / N1;
    __device__ __forceinline__ static int pos(int k) { return N2 * (k % N1) + k / N1; }
    __device__ __forceinline__ static int freq(int p) { return p / N2 + N1 * (p % N2); }
};

// n / d for 0 <= n < 2^22 and a block-invariant d >= 1 (inv = 1.0f / d):
// the float quotient is within one of the truth, one correction step.
__device__ __forceinline__ int div_inv(int n, int d, float inv) {
    int q = __float2int_rz((float)n * inv);
    const int r = n - q * d;
    if (r >= d) ++q;
    else if (r < 0) --q;
    return q;
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
                float2 w = __ldg(tw + Tw<N>::off + n2 * k1 * Tw<N>::stride);
                if (INV) w.y = -w.y;
                a[k1] = c_mul(a[k1], w);
            }
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) st(c, N2 * k1 + n2, a[k1]);
        }
    }
}

// SYNCW: a warp barrier between the loads and the stores of every item, so
// that fin may overwrite elements other lanes of the warp load (in place,
// with every transform's items inside one warp: count * N1 a multiple of 32
// and N1 dividing 32, so that all lanes of a warp run the same iterations).
template <int N, bool INV, bool CFAST, class LD, class FIN, bool SYNCW = false>
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
        if (SYNCW) __syncwarp();
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) fin(c, k1 + N1 * k2, N2 * k1 + k2, a[k2]);
    }
}

}  // namespace hpf_fft

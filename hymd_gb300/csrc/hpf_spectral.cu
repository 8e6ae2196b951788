// Fused spectral passes of the particle-field force: the paint's fixed-point
// accumulators -> filtered gradient force mesh in three kernels, with this
// library's own shared-memory FFTs (hpf_fft.cuh) instead of cuFFT.
//
// Reference sequence (paths inside the HyMD project): update_field
// hymd/field.py:428-616 (phi -> r2c -> H -> c2r -> v_ext -> r2c -> -i k H ->
// c2r), which for quadratic functionals is the single k-space map
//   F_{t,d}(k) = -i k'_d H(k)^2 (Q phi(k))_t / M  (+ the b_t term at k = 0),
// evaluated as in the library-FFT path (hpf_field.cu, k_kspace_force).
//
// Layouts are the library path's: real grids [g][x][y][z], half spectra
// [g][x][y][kz] with kz in [0, n2/2].  For meshes with n0 in {8..256 powers
// of two, 24, 48, 96, 192} and (n1, n2) both powers of two in 16..128 or
// both 24, 48 or 96 (the kernels are instantiated per size):
//   A  k_spec_fwd    one block per (type, x) plane: read the int64
//      accumulators (and clear them), scale to density, r2c along z (a
//      length-n2/2 complex transform and the usual split of even and odd
//      samples), c2c along y; write the plane of the half spectrum.
//   B  k_spec_kspace one block per tile of W (y, kz) columns: c2c along x of
//      the T density columns, the k-space map above and the Parseval sums of
//      the energy and pressure, inverse c2c along x of two columns per type,
//      -i k'_x v and v (the y and z forces -i k'_y v, -i k'_z v differ from
//      v by factors constant along x, applied in pass C).
//   C  k_spec_inv    one block per (force grid, x) plane: inverse c2c along
//      y, c2r along z; write the real plane.
// Each transform's first step reads its inputs from global memory (or
// computes them) and its second step writes global memory; shared memory
// holds only the data between steps.
// Each element is read and written once per pass; the intermediates of a
// 64^3 mesh stay in L2.  The FFTs are unnormalised as cuFFT's, so the
// k-space map is the same expression.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "hpf_fft.cuh"
#include "hpf_internal.cuh"

using namespace hpf_fft;

namespace {

constexpr int kSpecThreads = 256;
constexpr int kSpecWarps = kSpecThreads / 32;
constexpr int kSpecMaxT = 8;  // types handled by the fused path
constexpr size_t kSpecMaxSmem = 200 * 1024;
constexpr size_t kSpecTileSmem = 104 * 1024;

struct SpecGeom {
    int n0, n1, n2, h, nzc;  // h = n2 / 2, nzc = h + 1
    int W, ws;               // columns per k-space tile, log2 W
    int ts;                  // stride of a grid's block in a k-space tile (float2)
    int64_t M, Mc;
};

struct SpecScale {
    float s[kSpecMaxT + 1];
};

// Wavevector data of the W columns (y, kz) of a k-space tile.
struct ColInfo {
    float ky, kz, gy, gz, wk;
    int origin;  // column (0, 0): with kx = 0 the k = 0 mode
};

__device__ __forceinline__ void tile_columns(ColInfo* col, const SpecGeom& g, int j0,
                                             const BoxState* bs) {
    for (int w = threadIdx.x; w < g.W; w += blockDim.x) {
        const int j = j0 + w;
        const int iy = j / g.nzc, iz = j - iy * g.nzc;
        const int my = iy <= g.n1 / 2 ? iy : iy - g.n1;
        ColInfo ci;
        ci.ky = my * bs->kf[1];
        ci.kz = iz * bs->kf[2];
        // gradient wavevector: zero at the Nyquist index of each axis
        ci.gy = iy == g.n1 / 2 ? 0.0f : ci.ky;
        ci.gz = iz == g.h ? 0.0f : ci.kz;
        // half-spectrum multiplicity for Parseval sums
        ci.wk = (iz == 0 || iz == g.h) ? 1.0f : 2.0f;
        ci.origin = j == 0;
        col[w] = ci;
    }
}

// ------------------------------------------------------------ pass A ---
// Plane layout (passes A and C): row r of the (y, z) plane at
// r * plane_ls + r / N2y, N2y the y transform's second-step length (one
// slot of skew per block of N2y rows, so that the y transforms' accesses
// that run from column h of one row block into column 0 of the next land
// in consecutive banks).  Two layouts share a row, one after the other:
//   - between the two steps of the z transform, position p at p + p / N2
//     (one pad after every N2 elements, N2 the z transform's second-step
//     length), so that the stride-N2 accesses of its second step fall in
//     distinct banks;
//   - around the y transform, column (kz) c at c: a 16-lane access to 16
//     consecutive columns, or to their mirror columns h - c, is then
//     conflict-free.
// The z transform's second step changes one into the other in place (its
// items per row lie in one warp: a warp barrier between loads and stores).
// plane_ls = 8 mod 16 (in float2) puts the two rows a 16-lane access of the
// z transform touches in complementary banks.  Without a second step
// (h <= 16) each lane owns a row: odd stride.
__host__ __device__ constexpr int plane_n2(int h) { return h / split1(h); }
__host__ __device__ constexpr int plane_ls(int h) {
    return plane_n2(h) > 1 ? ((h + h / plane_n2(h) + 1 + 7) / 16) * 16 + 8 : ((h + 1) | 1);
}
// start of row r of a plane of ny rows
template <int NY, int HZ>
__device__ __forceinline__ int plane_row(int r) {
    constexpr int N2y = NY / split1(NY);
    return r * plane_ls(HZ) + (N2y > 1 ? r / N2y : 0);
}

// One block per (grid, x) plane.  z: int64 accumulators (read and cleared)
// -> length-h complex transform of the even/odd pairs; y: the split into
// the half spectrum X[0..h] fused into the first step of the y transform;
// the y transform's second step writes the spectrum plane.
// blockIdx.y: the grid (type) of acc and spec; sc.s[that grid] scales it.
// FIX = false: the input is a real grid (fin, float[grids][M]) scaled by
// sc.s[grid] alone, read and left as it is (the accumulators are not used).
template <int NY, int HZ, bool FIX = true>
__global__ void __launch_bounds__(kSpecThreads, 2)
    k_spec_fwd(unsigned long long* __restrict__ acc, float2* __restrict__ spec, SpecGeom g,
               SpecScale sc, const BoxState* __restrict__ bs, const float2* __restrict__ tw,
               const float* __restrict__ fin = nullptr) {
    pdl_wait();
    extern __shared__ __align__(16) float2 sm[];
    constexpr int Ny = NY, H = HZ, Nzc = H + 1, Ls = plane_ls(H), PN = plane_n2(H);
    // twiddles exp(-2 pi i k / n2) of the even/odd split
    constexpr int zoff = Tw<2 * H>::off, step = Tw<2 * H>::stride;
    const int x = blockIdx.x, t = blockIdx.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    auto zs = [](int e) { return PN > 1 ? e + e / PN : e; };
    auto row0 = [](int r) { return plane_row<NY, HZ>(r); };
    const float s = FIX ? sc.s[t] * bs->inv_dV * kFixInv : sc.s[t];
    ulonglong2* a =
        FIX ? reinterpret_cast<ulonglong2*>(acc + (int64_t)t * g.M + (int64_t)x * Ny * (2 * H))
            : nullptr;
    const float2* af =
        FIX ? nullptr
            : reinterpret_cast<const float2*>(fin + (int64_t)t * g.M + (int64_t)x * Ny * (2 * H));
    float2* out = spec + (int64_t)t * g.Mc + (int64_t)x * Ny * Nzc;
    constexpr float inv_rows = 1.0f / (float)Ny, inv_cols = 1.0f / (float)Nzc;
    {
        // z (rows r = y)
        auto ld = [&](int r, int m) {
            if constexpr (FIX) {
                const ulonglong2 v = __ldcg(a + r * H + m);
                a[r * H + m] = make_ulonglong2(0ull, 0ull);
                return make_float2(fix_to_float((long long)v.x) * s,
                                   fix_to_float((long long)v.y) * s);
            } else {
                const float2 v = __ldg(af + r * H + m);
                return make_float2(v.x * s, v.y * s);
            }
        };
        auto st = [&](int r, int p, float2 v) { sm[row0(r) + zs(p)] = v; };
        // (no second step: positions are frequencies, in natural order)
        auto fin = [&](int r, int k, int p, float2 v) { sm[row0(r) + zs(p)] = v; };
        fft_step1<H, false, false>(Ny, inv_rows, ld, st, fin, tw);
        __syncthreads();
        // second step: frequency k to column k
        static_assert(PN == 1 || ((Ny * split1(H)) % 32 == 0 && 32 % split1(H) == 0),
                      "the z transform's second-step items of a row lie in one warp");
        auto ld2 = [&](int r, int p) { return sm[row0(r) + zs(p)]; };
        auto fin2 = [&](int r, int k, int p, float2 v) { sm[row0(r) + k] = v; };
        fft_step2<H, false, false, decltype(ld2), decltype(fin2), true>(Ny, inv_rows, ld2, fin2);
    }
    __syncthreads();
    // y, step 1 with the even/odd split: X[k] = E + w^k O, X[h-k] = conj(E -
    // w^k O), E = (Z[k] + conj Z[h-k]) / 2, O = -i (Z[k] - conj Z[h-k]) / 2.
    // Columns k and h-k read each other's Z and are overwritten in place:
    // lanes 0-15 take 16 columns q, lanes 16-31 their partners h - q (h for
    // q = 0), one row offset n2 per warp task, a warp barrier between the
    // loads and the stores.  X[k] goes where Z[k] was, X[h] to slot h.
    {
        constexpr int N1 = split1(Ny), N2 = Ny / N1;
        constexpr int pairs = H / 2 + 1, groups = (pairs + 15) / 16;
        for (int task = warp; task < groups * N2; task += kSpecWarps) {
            const int gq = task / N2, n2 = task - gq * N2;
            const int q = gq * 16 + (lane & 15), side = lane >> 4;
            const bool active = q < pairs && !(side && q == H / 2);
            const int c = !active ? 0 : (side ? (q == 0 ? H : H - q) : q);
            const int kk = c == H ? 0 : c;
            const int pk = kk, pp = kk == 0 ? pk : H - kk;
            const float2 w = __ldg(tw + zoff + kk * step);
            float2 v[N1];
#pragma unroll
            for (int i = 0; i < N1; ++i) {
                const float2* row = sm + row0(N2 * i + n2);
                const float2 zk = row[pk], zp = row[pp];
                const float2 E = make_float2(0.5f * (zk.x + zp.x), 0.5f * (zk.y - zp.y));
                const float2 O = make_float2(0.5f * (zk.y + zp.y), -0.5f * (zk.x - zp.x));
                const float2 wO = c_mul(O, w);
                v[i] = c == H ? make_float2(E.x - wO.x, wO.y - E.y) : c_add(E, wO);
            }
            reg_fft<N1, false>(v);
            if (N2 > 1) {
#pragma unroll
                for (int k1 = 1; k1 < N1; ++k1)
                    v[k1] = c_mul(v[k1], __ldg(tw + Tw<Ny>::off + n2 * k1 * Tw<Ny>::stride));
            }
            __syncwarp();
            if (active) {
#pragma unroll
                for (int k1 = 0; k1 < N1; ++k1) sm[row0(N2 * k1 + n2) + c] = v[k1];
            }
            __syncwarp();
        }
        __syncthreads();
        if (N2 > 1) {
            // y, step 2: the spectrum plane, row ky = k1 + N1 k2
            auto ld2 = [&](int cc, int p) { return sm[row0(p) + cc]; };
            auto fin2 = [&](int cc, int ky, int p, float2 v2) { out[ky * Nzc + cc] = v2; };
            fft_step2<Ny, false, true>(Nzc, inv_cols, ld2, fin2);
        } else {
            // whole y transform in step 1: rows in natural order
            for (int ky = warp; ky < Ny; ky += kSpecWarps)
                for (int cc = lane; cc < Nzc; cc += 32) out[ky * Nzc + cc] = sm[row0(ky) + cc];
        }
    }
    pdl_trigger();
}

// ------------------------------------------------------------ pass B ---
// One block per tile of W (y, kz) columns: x transform of the T density
// columns (step 1 reads the spectrum planes), then the inverse x transforms
// of two columns per type (-i g_x v_t and v_t, v_t from the k-space map
// applied in place to the transformed densities), whose second step writes
// the output spectra.  Tile layout [grid][x][w], grids g.ts apart.
template <int N>
__global__ void __launch_bounds__(kSpecThreads, 2)
    k_spec_kspace(const float2* __restrict__ phi, float2* __restrict__ force, SpecGeom g, int T,
                  const BoxState* __restrict__ bs, const Functional* __restrict__ fun,
                  const float2* __restrict__ tw, double* sums, double* partials,
                  unsigned int* ticket) {
    pdl_wait();
    extern __shared__ __align__(16) float2 sm[];
    __shared__ float sQ[kSpecMaxT * kSpecMaxT], sb[kSpecMaxT];
    __shared__ ColInfo col[16];
    const int W = g.W, ws = g.ws, TS = g.ts;
    const int64_t plane = (int64_t)g.n1 * g.nzc;  // stride of x in a half spectrum
    const int j0 = blockIdx.x * W;
    float2* in = sm;            // [T][Nx][W]
    float2* out = sm + T * TS;  // [2T][Nx][W]
    for (int e = threadIdx.x; e < T * T; e += blockDim.x)
        sQ[(e / T) * kSpecMaxT + e % T] = fun->Q[e];
    for (int e = threadIdx.x; e < T; e += blockDim.x) sb[e] = fun->b[e];
    tile_columns(col, g, j0, bs);
    using fx = Idx<N>;
    const float kf0 = bs->kf[0];
    const float invM = (float)bs->inv_M;
    const float s2h = fun->sigma2_half;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const int cin = T * W, cout = 2 * T * W;
    const float inv_cin = 1.0f / (float)cin, inv_cout = 1.0f / (float)cout;
    {
        constexpr int N1 = split1(N), N2 = N / N1;
        auto at_in = [&](int c, int e) -> float2& { return in[(c >> ws) * TS + e * W + (c & (W - 1))]; };
        auto at_out = [&](int c, int e) -> float2& { return out[(c >> ws) * TS + e * W + (c & (W - 1))]; };
        // forward x transform of the densities
        auto ld = [&](int c, int n) {
            return __ldg(phi + (int64_t)(c >> ws) * g.Mc + n * plane + j0 + (c & (W - 1)));
        };
        auto st = [&](int c, int p, float2 v) { at_in(c, p) = v; };
        auto fin = [&](int c, int k, int p, float2 v) { at_in(c, p) = v; };
        __syncthreads();  // sQ, sb, col
        fft_step1<N, false, true>(cin, inv_cin, ld, st, fin, tw);
        __syncthreads();
        auto ld2 = [&](int c, int p) { return at_in(c, p); };
        fft_step2<N, false, true>(cin, inv_cin, ld2, fin);
        __syncthreads();
        // k-space map in place, one thread per mode (p, w): v_t = H^2 (Q
        // phi)_t / M (+ H b_t at k = 0) over the T densities phi; and the
        // Parseval sums of the energy and the pressure, q = sum_t ph_t . (Q
        // ph)_t with ph = H phi / M, weighted by the multiplicity.  The type
        // count is a compile-time constant of each variant (its loops fully
        // unrolled to T^2 products).
        auto map = [&](auto tc) {
            constexpr int TT = decltype(tc)::value;
            for (int e = threadIdx.x; e < N * W; e += blockDim.x) {
                const int p = e >> ws, w = e & (W - 1);
                const int ix = fx::freq(p);
                const ColInfo ci = col[w];
                const bool origin = ix == 0 && ci.origin;
                const float kx = (ix <= N / 2 ? ix : ix - N) * kf0;
                const float k2 = kx * kx + ci.ky * ci.ky + ci.kz * ci.kz;
                const float Hk = expf(-s2h * k2);
                const float hm = Hk * invM;
                float2 ph[TT];
#pragma unroll
                for (int jj = 0; jj < TT; ++jj) ph[jj] = in[jj * TS + p * W + w];
                float qq = 0.0f;
#pragma unroll
                for (int tt = 0; tt < TT; ++tt) {
                    float2 u = make_float2(0.0f, 0.0f);
#pragma unroll
                    for (int jj = 0; jj < TT; ++jj) {
                        const float Qtj = sQ[tt * kSpecMaxT + jj];
                        u.x = fmaf(Qtj, ph[jj].x, u.x);
                        u.y = fmaf(Qtj, ph[jj].y, u.y);
                    }
                    qq = fmaf(ph[tt].x, u.x, fmaf(ph[tt].y, u.y, qq));
                    float2 v = make_float2(Hk * hm * u.x, Hk * hm * u.y);
                    if (origin) v.x += Hk * sb[tt];
                    in[tt * TS + p * W + w] = v;
                }
                if (sums && !origin) {
                    const float wq = ci.wk * qq * hm * hm;
                    acc[0] += wq;
                    acc[1] = fmaf(wq, kx * kx, acc[1]);
                    acc[2] = fmaf(wq, ci.ky * ci.ky, acc[2]);
                    acc[3] = fmaf(wq, ci.kz * ci.kz, acc[3]);
                }
            }
        };
        switch (T) {
            case 1: map(IntC<1>()); break;
            case 2: map(IntC<2>()); break;
            case 3: map(IntC<3>()); break;
            case 4: map(IntC<4>()); break;
            case 5: map(IntC<5>()); break;
            case 6: map(IntC<6>()); break;
            case 7: map(IntC<7>()); break;
            default: map(IntC<8>()); break;
        }
        __syncthreads();
        // inverse x transforms, step 1; item (grid 2 to + e, w, n2): e = 0
        // -i g_x v_to (the x force), e = 1 v_to itself (the y and z forces,
        // -i g_y v and -i g_z v, are formed from it in pass C: g_y and g_z
        // do not vary along x)
        const int items = cout * N2;
        for (int it = threadIdx.x; it < items; it += blockDim.x) {
            const int n2 = N2 == 1 ? 0 : div_inv(it, cout, inv_cout);
            const int c = it - n2 * cout;
            const int gq = c >> ws, w = c & (W - 1);
            const int to = gq >> 1, e = gq & 1;
            const float2* vt = in + to * TS + w;
            float2 a[N1];
#pragma unroll
            for (int i = 0; i < N1; ++i) {
                const int ix = N2 * i + n2;
                const float2 v = vt[fx::pos(ix) * W];
                const float gx = ix == N / 2 ? 0.0f : (ix <= N / 2 ? ix : ix - N) * kf0;
                a[i] = e ? v : make_float2(gx * v.y, -gx * v.x);
            }
            reg_fft<N1, true>(a);
            if (N2 > 1) {
#pragma unroll
                for (int k1 = 1; k1 < N1; ++k1) {
                    const float2 tw1 = __ldg(tw + Tw<N>::off + n2 * k1 * Tw<N>::stride);
                    a[k1] = c_mul(a[k1], make_float2(tw1.x, -tw1.y));
                }
            }
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) at_out(c, N2 * k1 + n2) = a[k1];
        }
        __syncthreads();
        // inverse x transforms, step 2: the force spectra
        auto ldo = [&](int c, int p) { return at_out(c, p); };
        auto fino = [&](int c, int xx, int p, float2 v2) {
            force[(int64_t)(c >> ws) * g.Mc + xx * plane + j0 + (c & (W - 1))] = v2;
        };
        if (N2 > 1) {
            fft_step2<N, true, true>(cout, inv_cout, ldo, fino);
        } else {
            for (int e = threadIdx.x; e < cout * N; e += blockDim.x) {
                const int xx = div_inv(e, cout, inv_cout), c = e - xx * cout;
                fino(c, xx, xx, at_out(c, xx));
            }
        }
    }
    pdl_trigger();
    if (sums) grid_reduce_store_f<4, kSpecThreads>(acc, partials, ticket, sums);
}

// PIC_Spectral variant of pass B (hymd/field.py:241-403, the library path's
// k_kspace_pic): one charge-density column set in, psi = 4 pi f H rho / k^2
// (k^2 = 1 at k = 0) out as -i k'_x psi (grid 0) and psi (grid 1), pass C
// forming psi and the field components -i k'_d psi from them; sum of
// w_k rho(k).psi(k) over the half spectrum into sums[0].
template <int N>
__global__ void __launch_bounds__(kSpecThreads, 2)
    k_spec_kspace_pic(const float2* __restrict__ rho, float2* __restrict__ out_spec, SpecGeom g,
                      const BoxState* __restrict__ bs, const Functional* __restrict__ fun,
                      float four_pi_fac, const float2* __restrict__ tw,
                      double* sums, double* partials, unsigned int* ticket, int filter) {
    pdl_wait();
    extern __shared__ __align__(16) float2 sm[];
    __shared__ ColInfo col[16];
    const int W = g.W, ws = g.ws, TS = g.ts;
    const int64_t plane = (int64_t)g.n1 * g.nzc;
    const int j0 = blockIdx.x * W;
    float2* in = sm;        // [Nx][W]
    float2* out = sm + TS;  // [2][Nx][W]: -i g_x psi, psi
    tile_columns(col, g, j0, bs);
    using fx = Idx<N>;
    const float kf0 = bs->kf[0];
    const float invM = (float)bs->inv_M;
    const float s2h = fun->sigma2_half;
    float acc[1] = {0.0f};
    const int cout = 2 * W;
    const float inv_w = 1.0f / (float)W, inv_cout = 1.0f / (float)cout;
    {
        constexpr int N1 = split1(N), N2 = N / N1;
        auto ld = [&](int c, int n) { return __ldg(rho + n * plane + j0 + c); };
        auto st = [&](int c, int p, float2 v) { in[p * W + c] = v; };
        auto fin = [&](int c, int k, int p, float2 v) { in[p * W + c] = v; };
        __syncthreads();  // col
        fft_step1<N, false, true>(W, inv_w, ld, st, fin, tw);
        __syncthreads();
        auto ld2 = [&](int c, int p) { return in[p * W + c]; };
        fft_step2<N, false, true>(W, inv_w, ld2, fin);
        __syncthreads();
        // item (grid e, w, n2): psi = 4 pi f H rho / k^2; e = 0 -i g_x psi
        // (E_x), e = 1 psi (psi, and E_y, E_z formed in pass C)
        const int items = cout * N2;
        for (int it = threadIdx.x; it < items; it += blockDim.x) {
            const int n2 = N2 == 1 ? 0 : div_inv(it, cout, inv_cout);
            const int c = it - n2 * cout;
            const int e = c >> ws, w = c & (W - 1);
            const ColInfo ci = col[w];
            float2 a[N1];
#pragma unroll
            for (int i = 0; i < N1; ++i) {
                const int ix = N2 * i + n2;
                const float kx = (ix <= N / 2 ? ix : ix - N) * kf0;
                float k2 = kx * kx + ci.ky * ci.ky + ci.kz * ci.kz;
                const float Hk = filter ? expf(-s2h * k2) : 1.0f;
                if (ix == 0 && ci.origin) k2 = 1.0f;  // k.normp(p=2, zeromode=1)
                const float2 r = in[fx::pos(ix) * W + w];
                const float2 rq = make_float2(r.x * invM, r.y * invM);
                const float sc = four_pi_fac * Hk / k2;
                const float2 v = make_float2(rq.x * sc, rq.y * sc);
                if (sums && e == 0)
                    acc[0] = fmaf(ci.wk, fmaf(rq.x, v.x, rq.y * v.y), acc[0]);
                const float gx = ix == N / 2 ? 0.0f : kx;
                a[i] = e ? v : make_float2(gx * v.y, -gx * v.x);
            }
            reg_fft<N1, true>(a);
            if (N2 > 1) {
#pragma unroll
                for (int k1 = 1; k1 < N1; ++k1) {
                    const float2 tw1 = __ldg(tw + Tw<N>::off + n2 * k1 * Tw<N>::stride);
                    a[k1] = c_mul(a[k1], make_float2(tw1.x, -tw1.y));
                }
            }
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) out[e * TS + (N2 * k1 + n2) * W + w] = a[k1];
        }
        __syncthreads();
        auto at_out = [&](int c, int q) -> float2& { return out[(c >> ws) * TS + q * W + (c & (W - 1))]; };
        auto ldo = [&](int c, int p) { return at_out(c, p); };
        auto fino = [&](int c, int xx, int p, float2 v2) {
            out_spec[(int64_t)(c >> ws) * g.Mc + xx * plane + j0 + (c & (W - 1))] = v2;
        };
        if (N2 > 1) {
            fft_step2<N, true, true>(cout, inv_cout, ldo, fino);
        } else {
            for (int q = threadIdx.x; q < cout * N; q += blockDim.x) {
                const int xx = div_inv(q, cout, inv_cout), c = q - xx * cout;
                fino(c, xx, xx, at_out(c, xx));
            }
        }
    }
    pdl_trigger();
    if (sums) grid_reduce_store_f<1, kSpecThreads>(acc, partials, ticket, sums);
}

// ------------------------------------------------------------ pass C ---
// One block per (force grid, x) plane: inverse y transform (step 1 reads the
// spectrum plane; columns kz in natural order), then the inverse z transform
// of the even/odd packing
//   Z'[m] = A + i v B, A = X[m] + conj X[h-m], B = X[m] - conj X[h-m],
//   v = exp(+2 pi i m / n2),
// whose length-h inverse gives the even (real) and odd (imaginary) samples;
// the packing is computed in the z transform's first step (rows handled by
// one warp each, since X[m] and X[h-m] are overwritten in place) and its
// second step writes the real plane.
// Output grid gi (density: 3 t + d; PIC: psi, E_x, E_y, E_z) comes from
// pass B's grid src: -i g_x v (x force) as is, v times -i g_y (a function
// of the row ky) or -i g_z (of the column kz) for the y and z forces, v as
// is for psi.
template <int NY, int HZ>
__global__ void __launch_bounds__(kSpecThreads, 2)
    k_spec_inv(const float2* __restrict__ spec, float* __restrict__ grid, SpecGeom g,
               const BoxState* __restrict__ bs, const float2* __restrict__ tw, int first,
               int pic) {
    pdl_wait();
    extern __shared__ __align__(16) float2 sm[];
    constexpr int Ny = NY, H = HZ, Nzc = H + 1, Ls = plane_ls(H), PN = plane_n2(H);
    constexpr int zoff = Tw<2 * H>::off, step = Tw<2 * H>::stride;
    const int x = blockIdx.x, gi = blockIdx.y + first;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    using fy = Idx<Ny>;
    auto zs = [](int e) { return PN > 1 ? e + e / PN : e; };
    auto row0 = [](int r) { return plane_row<NY, HZ>(r); };
    int src, mul;  // mul: 0 none, 1 -i g_y, 2 -i g_z
    if (pic) {
        src = gi == 1 ? 0 : 1;
        mul = gi == 2 ? 1 : (gi == 3 ? 2 : 0);
    } else {
        const int t = gi / 3, d = gi - 3 * t;
        src = 2 * t + (d > 0);
        mul = d;
    }
    const float kf1 = bs->kf[1], kf2 = bs->kf[2];
    const float2* in = spec + (int64_t)src * g.Mc + (int64_t)x * Ny * Nzc;
    float2* out = reinterpret_cast<float2*>(grid + ((int64_t)gi * g.n0 + x) * Ny * (2 * H));
    constexpr float inv_rows = 1.0f / (float)Ny, inv_cols = 1.0f / (float)Nzc;
    {
        // y: rows left at FftIdx positions of y
        auto ld = [&](int c, int n) { return __ldg(in + n * Nzc + c); };
        auto pre = [&](int c, int n2, auto& a) {
            constexpr int N1 = split1(Ny), N2 = Ny / N1;
            if (mul == 0) return;
#pragma unroll
            for (int i = 0; i < N1; ++i) {
                const int n = N2 * i + n2;
                const float gd = mul == 1
                                     ? (n == Ny / 2 ? 0.0f : (n <= Ny / 2 ? n : n - Ny) * kf1)
                                     : (c == H ? 0.0f : c * kf2);
                a[i] = make_float2(gd * a[i].y, -gd * a[i].x);
            }
        };
        auto st = [&](int c, int p, float2 v) { sm[row0(p) + c] = v; };
        auto fin = [&](int c, int k, int p, float2 v) { sm[row0(p) + c] = v; };
        fft_step1<Ny, true, true>(Nzc, inv_cols, ld, st, fin, tw, pre);
        __syncthreads();
        auto ld2 = [&](int c, int p) { return sm[row0(p) + c]; };
        fft_step2<Ny, true, true>(Nzc, inv_cols, ld2, fin);
    }
    __syncthreads();
    {
        constexpr int N1 = split1(H), N2 = H / N1;
        constexpr int RPW = 32 / N2;  // rows per warp
        for (int r0 = warp * RPW; r0 < Ny; r0 += kSpecWarps * RPW) {
            const int r = r0 + lane / N2, n2 = lane % N2;
            const bool active = lane < RPW * N2 && r < Ny;
            float2* row = sm + row0(active ? r : 0);
            float2 a[N1];
#pragma unroll
            for (int i = 0; i < N1; ++i) {
                const int m = N2 * i + n2;
                const float2 xk = row[m], xp = row[H - m];
                const float2 A = make_float2(xk.x + xp.x, xk.y - xp.y);
                const float2 B = make_float2(xk.x - xp.x, xk.y + xp.y);
                const float2 w = __ldg(tw + zoff + m * step);
                const float2 vB = c_mul(B, make_float2(w.x, -w.y));
                a[i] = make_float2(A.x - vB.y, A.y + vB.x);
            }
            reg_fft<N1, true>(a);
            if (N2 > 1) {
#pragma unroll
                for (int k1 = 1; k1 < N1; ++k1) {
                    const float2 tw1 = __ldg(tw + Tw<H>::off + n2 * k1 * Tw<H>::stride);
                    a[k1] = c_mul(a[k1], make_float2(tw1.x, -tw1.y));
                }
            }
            __syncwarp();
            if (active) {
#pragma unroll
                for (int k1 = 0; k1 < N1; ++k1) row[zs(N2 * k1 + n2)] = a[k1];
            }
            __syncwarp();
        }
        __syncthreads();
        auto fin = [&](int r, int m, int p, float2 v) { out[fy::freq(r) * H + m] = v; };
        if (N2 > 1) {
            auto ld2 = [&](int r, int p) { return sm[row0(r) + zs(p)]; };
            fft_step2<H, true, false>(Ny, inv_rows, ld2, fin);
        } else {
            for (int r = warp; r < Ny; r += kSpecWarps)
                for (int m = lane; m < H; m += 32) fin(r, m, m, sm[row0(r) + m]);
        }
    }
    pdl_trigger();
}

// The k-space kernels are instantiated per x length (their register
// transforms are sized by it); f(kernel pointer) for this mesh.
template <class F>
int with_kspace(int nx, F f) {
    switch (nx) {
        case 8: return f(k_spec_kspace<8>, k_spec_kspace_pic<8>);
        case 16: return f(k_spec_kspace<16>, k_spec_kspace_pic<16>);
        case 32: return f(k_spec_kspace<32>, k_spec_kspace_pic<32>);
        case 64: return f(k_spec_kspace<64>, k_spec_kspace_pic<64>);
        case 128: return f(k_spec_kspace<128>, k_spec_kspace_pic<128>);
        case 256: return f(k_spec_kspace<256>, k_spec_kspace_pic<256>);
        case 24: return f(k_spec_kspace<24>, k_spec_kspace_pic<24>);
        case 48: return f(k_spec_kspace<48>, k_spec_kspace_pic<48>);
        case 96: return f(k_spec_kspace<96>, k_spec_kspace_pic<96>);
        case 192: return f(k_spec_kspace<192>, k_spec_kspace_pic<192>);
        default: return HPF_ERR_ARG;
    }
}

int ilog2_host(int n) {
    int s = 0;
    while ((1 << s) < n) ++s;
    return s;
}

int tile_pad(int W) { return W < 16 ? W : 0; }

SpecGeom spec_geom(const hpf_ctx* c, int W) {
    SpecGeom g;
    g.n0 = c->n0;
    g.n1 = c->n1;
    g.n2 = c->n2;
    g.h = c->n2 / 2;
    g.nzc = g.h + 1;
    g.W = W;
    g.ws = ilog2_host(g.W > 0 ? g.W : 1);
    g.ts = c->n0 * g.W + tile_pad(g.W);
    g.M = c->M;
    g.Mc = c->Mc;
    return g;
}

size_t plane_smem(const hpf_ctx* c) {
    // rows, then the skew of the last row block (at most split1(n1) - 1 slots)
    return sizeof(float2) * ((size_t)c->n1 * plane_ls(c->n2 / 2) + split1(c->n1));
}

// The plane kernels are instantiated per (n1, n2 / 2): n1 and n2 in
// {16, 32, 64, 128}, and the cubic 24, 48, 96.  f(fwd kernel, inv kernel)
// for this mesh.
template <class F>
int with_planes(int n1, int h, F f) {
#define HPF_PLANE(NY, HZ)   \
    if (n1 == NY && h == HZ) \
        return f(k_spec_fwd<NY, HZ>, k_spec_inv<NY, HZ>, k_spec_fwd<NY, HZ, false>);
#define HPF_PLANES(NY) HPF_PLANE(NY, 8) HPF_PLANE(NY, 16) HPF_PLANE(NY, 32) HPF_PLANE(NY, 64)
    HPF_PLANES(16)
    HPF_PLANES(32)
    HPF_PLANES(64)
    HPF_PLANES(128)
    HPF_PLANE(24, 12)
    HPF_PLANE(48, 24)
    HPF_PLANE(96, 48)
#undef HPF_PLANES
#undef HPF_PLANE
    return HPF_ERR_ARG;
}
// a k-space tile: T density blocks in + 2T out, or (pic) 1 charge block in
// + 2 out
size_t tile_smem(const hpf_ctx* c, int W, bool pic = false) {
    const int blocks = pic ? 3 : 3 * c->T;
    return sizeof(float2) * (size_t)blocks * (c->n0 * W + tile_pad(W));
}

// The widest tile of W in {16, 8, 4} columns that divides n1, fits the
// shared-memory budget and leaves a tile for every SM (4 when none does).
// The charge pass takes it for itself: with one grid in, narrower tiles
// leave most of a block's threads without an item in the x transforms.
int widest_tile(const hpf_ctx* c, bool pic) {
    const int64_t cols = (int64_t)c->n1 * (c->n2 / 2 + 1);
    int W = 16;
    while (W > 4 && (c->n1 % W != 0 || tile_smem(c, W, pic) > kSpecTileSmem || cols / W < 152))
        W >>= 1;
    return W;
}

}  // namespace

// Whether the fused passes apply to this context's mesh and type count.
bool spectral_eligible(const hpf_ctx* c) {
    if (c->T > kSpecMaxT) return false;
    if (with_kspace(c->n0, [](auto, auto) { return HPF_OK; }) != HPF_OK) return false;
    if (plane_smem(c) > kSpecMaxSmem) return false;
    if (with_planes(c->n1, c->n2 / 2, [](auto, auto, auto) { return HPF_OK; }) != HPF_OK) return false;
    return tile_smem(c, 4) <= kSpecTileSmem;
}

// Whether pass B can run tiles of W columns on this context: W in {4, 8,
// 16} (the tile's column table holds 16), dividing n1 (so that the n1 * (n2/2
// + 1) columns split into whole tiles), within the shared-memory budget.
bool spectral_tile_ok(const hpf_ctx* c, int W) {
    if (W != 4 && W != 8 && W != 16) return false;
    return c->n1 % W == 0 && tile_smem(c, W) <= kSpecTileSmem;
}

// Select the k-space tile width (the autotuner's knob); the partials were
// sized for the narrowest tile at setup.
int spectral_set_tile(hpf_ctx* c, int W) {
    if (!c->spec_ok || !spectral_tile_ok(c, W)) return HPF_ERR_ARG;
    c->spec_W = W;
    c->spec_tiles = (int)((int64_t)c->n1 * (c->n2 / 2 + 1) / W);
    return HPF_OK;
}

// Twiddle table, tile width and reduction scratch (at context creation).
int spectral_setup(hpf_ctx* c) {
    if (!spectral_eligible(c)) return HPF_OK;
    // default: the widest tile that leaves a block for every SM
    const int W = widest_tile(c, false);
    const int64_t cols = (int64_t)c->n1 * (c->n2 / 2 + 1);
    if (!spectral_tile_ok(c, W)) return HPF_OK;
    c->spec_W = W;
    c->spec_tiles = (int)(cols / W);
    c->spec_W_pic = widest_tile(c, true);
    c->spec_tiles_pic = (int)(cols / c->spec_W_pic);
    float2 h_tw[kTableTotal];
    for (int m = 0; m < kTable2; ++m) {
        const double a = -2.0 * 3.14159265358979323846 * (double)m / (double)kTable2;
        h_tw[m] = make_float2((float)cos(a), (float)sin(a));
    }
    for (int m = 0; m < kTable3; ++m) {
        const double a = -2.0 * 3.14159265358979323846 * (double)m / (double)kTable3;
        h_tw[kTable2 + m] = make_float2((float)cos(a), (float)sin(a));
    }
    if (cudaMalloc(&c->d_tw, sizeof(h_tw)) != cudaSuccess) return HPF_ERR_CUDA;
    if (cudaMemcpy(c->d_tw, h_tw, sizeof(h_tw), cudaMemcpyHostToDevice) != cudaSuccess)
        return HPF_ERR_CUDA;
    // partials: 4 values x tiles (double-float pairs), then the ticket; room
    // for the narrowest tile, so that the width can change later
    c->spec_max_tiles = (int)(cols / 4);
    const size_t words = spectral_ws_words(c);
    if (cudaMalloc(&c->d_spec_ws, sizeof(double) * words) != cudaSuccess) return HPF_ERR_CUDA;
    if (cudaMemset(c->d_spec_ws, 0, sizeof(double) * words) != cudaSuccess) return HPF_ERR_CUDA;
    // the kernels' shared-memory ceilings are process-wide attributes: set
    // them to the largest size any context may launch with
    const int ps = (int)kSpecMaxSmem, ts = (int)kSpecTileSmem;
    if (with_planes(c->n1, c->n2 / 2, [&](auto kf, auto ki, auto kr) {
            return (cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, ps) !=
                        cudaSuccess ||
                    cudaFuncSetAttribute(ki, cudaFuncAttributeMaxDynamicSharedMemorySize, ps) !=
                        cudaSuccess ||
                    cudaFuncSetAttribute(kr, cudaFuncAttributeMaxDynamicSharedMemorySize, ps) !=
                        cudaSuccess)
                       ? HPF_ERR_CUDA
                       : HPF_OK;
        }) != HPF_OK ||
        with_kspace(c->n0, [&](auto kd, auto kp) {
            return (cudaFuncSetAttribute(kd, cudaFuncAttributeMaxDynamicSharedMemorySize, ts) !=
                        cudaSuccess ||
                    cudaFuncSetAttribute(kp, cudaFuncAttributeMaxDynamicSharedMemorySize, ts) !=
                        cudaSuccess)
                       ? HPF_ERR_CUDA
                       : HPF_OK;
        }) != HPF_OK)
        return HPF_ERR_CUDA;
    c->spec_fused = 1;
    c->spec_ok = 1;
    return HPF_OK;
}

size_t spectral_ws_words(const hpf_ctx* c) { return 4 * (size_t)c->spec_max_tiles + 8; }

// accumulators (T grids, painted) -> force mesh c->d_grid [3T][M]; sums as
// k_kspace_force's (out[0..3]) when non-null.
int spectral_field_force(hpf_ctx* c, const float* type_scale, double* sums, cudaStream_t st) {
    const SpecGeom g = spec_geom(c, c->spec_W);
    SpecScale sc;
    for (int t = 0; t < c->T; ++t) sc.s[t] = type_scale[t];
    const int ps = (int)plane_smem(c), ts = (int)tile_smem(c, g.W);
    if (with_planes(c->n1, c->n2 / 2, [&](auto kf, auto, auto) {
            return launch_pdl(kf, dim3(c->n0, c->T), kSpecThreads, ps, st, c->d_acc,
                              c->d_spec_phi, g, sc, c->d_box, c->d_tw, nullptr) == cudaSuccess
                       ? HPF_OK
                       : HPF_ERR_CUDA;
        }) != HPF_OK)
        return HPF_ERR_CUDA;
    double* part = c->d_spec_ws;
    unsigned int* tick = reinterpret_cast<unsigned int*>(c->d_spec_ws + 4 * (size_t)c->spec_max_tiles);
    int r = with_kspace(c->n0, [&](auto kd, auto) {
        return launch_pdl(kd, c->spec_tiles, kSpecThreads, ts, st, c->d_spec_phi, c->d_spec, g,
                          c->T, c->d_box, c->d_fun, c->d_tw, sums, part, tick) == cudaSuccess
                   ? HPF_OK
                   : HPF_ERR_CUDA;
    });
    if (r != HPF_OK) return r;
    HPF_LAUNCH_CHECK();
    if (with_planes(c->n1, c->n2 / 2, [&](auto, auto ki, auto) {
            return launch_pdl(ki, dim3(c->n0, 3 * c->T), kSpecThreads, ps, st, c->d_spec,
                              c->d_grid, g, c->d_box, c->d_tw, 0, 0) == cudaSuccess
                       ? HPF_OK
                       : HPF_ERR_CUDA;
        }) != HPF_OK)
        return HPF_ERR_CUDA;
    return HPF_OK;
}

// charge accumulator (slot T, painted), or the real grid real_in -> psi
// (grid 0, when want_psi) and E_d (grids 1..3) in b.grid; sums[0] as
// k_kspace_pic's when non-null.
int spectral_pic(hpf_ctx* c, const SpecBufs& b, float four_pi_fac, bool want_psi, double* sums,
                 cudaStream_t st, const float* real_in, bool filter) {
    const SpecGeom g = spec_geom(c, c->spec_W_pic);
    SpecScale sc;
    sc.s[0] = 1.0f;
    const int ps = (int)plane_smem(c), ts = (int)tile_smem(c, g.W, true);
    if (with_planes(c->n1, c->n2 / 2, [&](auto kf, auto, auto kr) {
            const cudaError_t e =
                real_in ? launch_pdl(kr, dim3(c->n0, 1), kSpecThreads, ps, st, nullptr,
                                     b.spec_phi, g, sc, c->d_box, c->d_tw, real_in)
                        : launch_pdl(kf, dim3(c->n0, 1), kSpecThreads, ps, st,
                                     c->d_acc + (int64_t)c->T * c->M, b.spec_phi, g, sc,
                                     c->d_box, c->d_tw, nullptr);
            return e == cudaSuccess ? HPF_OK : HPF_ERR_CUDA;
        }) != HPF_OK)
        return HPF_ERR_CUDA;
    double* part = b.ws;
    unsigned int* tick = reinterpret_cast<unsigned int*>(b.ws + 4 * (size_t)c->spec_max_tiles);
    int r = with_kspace(c->n0, [&](auto, auto kp) {
        return launch_pdl(kp, c->spec_tiles_pic, kSpecThreads, ts, st, b.spec_phi, b.spec, g,
                          c->d_box, c->d_fun, four_pi_fac, c->d_tw, sums, part, tick,
                          filter ? 1 : 0) == cudaSuccess
                   ? HPF_OK
                   : HPF_ERR_CUDA;
    });
    if (r != HPF_OK) return r;
    HPF_LAUNCH_CHECK();
    const int first = want_psi ? 0 : 1;
    if (with_planes(c->n1, c->n2 / 2, [&](auto, auto ki, auto) {
            return launch_pdl(ki, dim3(c->n0, 4 - first), kSpecThreads, ps, st, b.spec, b.grid,
                              g, c->d_box, c->d_tw, first, 1) == cudaSuccess
                       ? HPF_OK
                       : HPF_ERR_CUDA;
        }) != HPF_OK)
        return HPF_ERR_CUDA;
    return HPF_OK;
}

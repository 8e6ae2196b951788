/*
 * FP32 multi-core restatement of the per-step CPU work of HyMD's
 * particle-field path -- TEST INFRASTRUCTURE ONLY: the timed CPU baseline of
 * bench.py (and the tests that check it) load this; the CUDA library never
 * does.
 *
 * It follows the reference's sequence and float32 arithmetic (config.dtype
 * float32, pmesh "f4"):
 *   pm.paint / RealField.readout (CIC)     hymd/field.py:152-200, 573-575, 356-403
 *   apply(H), apply(-i k_d), Poisson map    hymd/field.py:576-616, 366-397
 *   v_ext[t](phi) for quadratic functionals hymd/hamiltonian.py:470-473
 *   integrate_velocity / integrate_position + wrap  hymd/integrator.py:9-73,
 *                                           hymd/main.py:830-887
 * with the mesh conventions of the FP64 oracle (oracle/field.py): nodes at
 * x = i h, r2c / M, c2r unnormalised, k_d = 2 pi m / L_d, zero gradient at a
 * Nyquist index.  The transforms themselves are scipy.fft's, called from
 * oracle/cpu_md.py.  OpenMP over all host cores stands in for the
 * reference's MPI ranks: paint into per-thread grids summed in a fixed order,
 * everything else split by particle or by mesh plane.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#else
static int omp_get_max_threads(void) { return 1; }
static int omp_get_thread_num(void) { return 0; }
#endif

static inline int64_t wrap_i(int64_t i, int64_t n) {
    i %= n;
    return i < 0 ? i + n : i;
}

int cpu_threads(void) { return omp_get_max_threads(); }

/* CIC paint of n particles into G grids of M = n0 n1 n2 float cells:
 * grid g(i) = grid_of ? grid_of[i] : 0 receives weight w_i =
 * (weight ? weight[i] : 1) * gscale[g(i)] times the 8 corner weights
 * (1 - |s - i|) per axis, s = x n / L.  out (float[G][M]) is overwritten.
 * Particles with grid_of[i] outside [0, G) are skipped. */
void cpu_paint(const float* pos, const int32_t* grid_of, const float* weight,
               const float* gscale, int64_t n, int G, int n0, int n1, int n2,
               const double* box, float* out) {
    const int64_t M = (int64_t)n0 * n1 * n2;
    const int nt = omp_get_max_threads();
    float* priv = (float*)calloc((size_t)nt * G * M, sizeof(float));
    const float s0 = (float)(n0 / box[0]), s1 = (float)(n1 / box[1]), s2 = (float)(n2 / box[2]);
#pragma omp parallel
    {
        float* g = priv + (int64_t)omp_get_thread_num() * G * M;
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            const int gi = grid_of ? grid_of[i] : 0;
            if (gi < 0 || gi >= G) continue;
            const float w = (weight ? weight[i] : 1.0f) * gscale[gi];
            if (w == 0.0f) continue;
            const float x = pos[3 * i] * s0, y = pos[3 * i + 1] * s1, z = pos[3 * i + 2] * s2;
            const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
            const float dx = x - fx, dy = y - fy, dz = z - fz;
            const int64_t ix = wrap_i((int64_t)fx, n0), iy = wrap_i((int64_t)fy, n1),
                          iz = wrap_i((int64_t)fz, n2);
            const int64_t jx = ix + 1 == n0 ? 0 : ix + 1, jy = iy + 1 == n1 ? 0 : iy + 1,
                          jz = iz + 1 == n2 ? 0 : iz + 1;
            float* gg = g + (int64_t)gi * M;
            const float wx[2] = {1.0f - dx, dx}, wy[2] = {1.0f - dy, dy}, wz[2] = {1.0f - dz, dz};
            const int64_t xs[2] = {ix, jx}, ys[2] = {iy, jy}, zs[2] = {iz, jz};
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b) {
                    float* row = gg + (xs[a] * n1 + ys[b]) * n2;
                    const float wab = w * wx[a] * wy[b];
                    row[zs[0]] += wab * wz[0];
                    row[zs[1]] += wab * wz[1];
                }
        }
    }
    const int64_t total = (int64_t)G * M;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < total; ++c) {
        float s = 0.0f;
        for (int t = 0; t < nt; ++t) s += priv[(int64_t)t * total + c];
        out[c] = s;
    }
    free(priv);
}

/* Readout of `ncomp` grid components per particle: out[i][d] =
 * scale_i * sum_corners W * grids[(g(i) * ncomp + d) * M + cell], with
 * g(i) = grid_of ? grid_of[i] : 0 and scale_i = scale ? scale[i] : 1. */
void cpu_readout(const float* grids, const float* pos, const int32_t* grid_of,
                 const float* scale, int64_t n, int ncomp, int n0, int n1, int n2,
                 const double* box, float* out) {
    const int64_t M = (int64_t)n0 * n1 * n2;
    const float s0 = (float)(n0 / box[0]), s1 = (float)(n1 / box[1]), s2 = (float)(n2 / box[2]);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const int gi = grid_of ? grid_of[i] : 0;
        const float x = pos[3 * i] * s0, y = pos[3 * i + 1] * s1, z = pos[3 * i + 2] * s2;
        const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
        const float dx = x - fx, dy = y - fy, dz = z - fz;
        const int64_t ix = wrap_i((int64_t)fx, n0), iy = wrap_i((int64_t)fy, n1),
                      iz = wrap_i((int64_t)fz, n2);
        const int64_t xs[2] = {ix, ix + 1 == n0 ? 0 : ix + 1};
        const int64_t ys[2] = {iy, iy + 1 == n1 ? 0 : iy + 1};
        const int64_t zs[2] = {iz, iz + 1 == n2 ? 0 : iz + 1};
        const float wx[2] = {1.0f - dx, dx}, wy[2] = {1.0f - dy, dy}, wz[2] = {1.0f - dz, dz};
        const float sc = scale ? scale[i] : 1.0f;
        for (int d = 0; d < ncomp; ++d) {
            const float* g = grids + ((int64_t)gi * ncomp + d) * M;
            float acc = 0.0f;
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b) {
                    const float* row = g + (xs[a] * n1 + ys[b]) * n2;
                    const float wab = wx[a] * wy[b];
                    acc += wab * (wz[0] * row[zs[0]] + wz[1] * row[zs[1]]);
                }
            out[3 * i + d] = sc * acc;
        }
    }
}

static inline float kval(int64_t m, int n, double L, int zero_nyquist) {
    if (zero_nyquist && (n % 2 == 0) && m == n / 2) return 0.0f;
    const int64_t mm = m < (n + 1) / 2 ? m : m - n;
    return (float)(6.283185307179586 / L * (double)mm);
}

/* Spectral maps on a half spectrum (complex64 as float pairs,
 * [n0][n1][n2/2+1]):
 *   mode 0: out = H(k) in                 (apply(hamiltonian.H))
 *   mode 1: out = -i k_d in               (force transfer, zero at Nyquist)
 *   mode 2: out = c in / |k|^2, k=0 -> 1  (Poisson, c = 4 pi k_e / eps)
 *   mode 3: out = -k_d^2 in               (Laplacian component)
 * H(k) = exp(-sigma^2 |k|^2 / 2) with the full |k|^2.  out may alias in. */
void cpu_kmap(const float* in, float* out, int n0, int n1, int n2, const double* box, int mode,
              int d, double sigma, double c) {
    const int64_t nh = n2 / 2 + 1;
#pragma omp parallel for schedule(static)
    for (int64_t x = 0; x < n0; ++x) {
        const float kx = kval(x, n0, box[0], 0), gx = kval(x, n0, box[0], 1);
        for (int64_t y = 0; y < n1; ++y) {
            const float ky = kval(y, n1, box[1], 0), gy = kval(y, n1, box[1], 1);
            const int64_t base = (x * n1 + y) * nh;
            for (int64_t z = 0; z < nh; ++z) {
                const float kz = kval(z, n2, box[2], 0), gz = kval(z, n2, box[2], 1);
                const float k2 = kx * kx + ky * ky + kz * kz;
                const float re = in[2 * (base + z)], im = in[2 * (base + z) + 1];
                float o_re, o_im;
                if (mode == 0) {
                    const float h = expf((float)(-0.5 * sigma * sigma) * k2);
                    o_re = h * re;
                    o_im = h * im;
                } else if (mode == 1) {
                    const float g = d == 0 ? gx : (d == 1 ? gy : gz);
                    o_re = g * im;
                    o_im = -g * re;
                } else if (mode == 2) {
                    const float den = (x == 0 && y == 0 && z == 0) ? 1.0f : k2;
                    o_re = (float)c * re / den;
                    o_im = (float)c * im / den;
                } else {
                    const float k = d == 0 ? kx : (d == 1 ? ky : kz);
                    o_re = -k * k * re;
                    o_im = -k * k * im;
                }
                out[2 * (base + z)] = o_re;
                out[2 * (base + z) + 1] = o_im;
            }
        }
    }
}

/* v = sum_j Q[t][j] phi_j + b[t] on M cells (v_ext of a quadratic
 * functional, hamiltonian.py:470-473). */
void cpu_vext(const float* phi, int T, int64_t M, const double* Qrow, double b, float* v) {
    float q[16];
    for (int j = 0; j < T && j < 16; ++j) q[j] = (float)Qrow[j];
    const float bf = (float)b;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < M; ++c) {
        float s = bf;
        for (int j = 0; j < T; ++j) s += q[j] * phi[(int64_t)j * M + c];
        v[c] = s;
    }
}

/* v += h * sum_f F_f / mass over nf force arrays (integrate_velocity), then
 * optionally r = mod(r + dt v, L) (integrate_position + the wrap of
 * main.py:837). */
void cpu_kick_drift(float* r, float* v, const float* const* forces, int nf, int64_t n,
                    double mass, double h, double dt, const double* box, int drift) {
    const float hm = (float)(h / mass), dtf = (float)dt;
    const float L[3] = {(float)box[0], (float)box[1], (float)box[2]};
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        for (int d = 0; d < 3; ++d) {
            float f = 0.0f;
            for (int q = 0; q < nf; ++q) f += forces[q][3 * i + d];
            float vv = v[3 * i + d] + hm * f;
            v[3 * i + d] = vv;
            if (drift) {
                float x = r[3 * i + d] + dtf * vv;
                x = fmodf(x, L[d]);
                if (x < 0.0f) x += L[d];
                r[3 * i + d] = x;
            }
        }
    }
}

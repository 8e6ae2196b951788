// Particle-field path of HyMD on GB300: mesh context, deterministic CIC
// paint, fused k-space pass, CIC readout, PIC_Spectral electrostatics.
//
// Reference behaviour (paths inside the HyMD project):
//   update_field            hymd/field.py:428-616
//   compute_field_force     hymd/field.py:152-200
//   update_field_force_q    hymd/field.py:241-403
//   comp_laplacian / comp_pressure  hymd/field.py:406-425, hymd/pressure.py:9-179
//
// All interaction functionals of the reference are quadratic in the filtered
// densities phi~ (hymd/hamiltonian.py:74-486), so v_ext = Q phi~ + b is a T x T
// linear map per wavevector.  The reference sequence
//   phi~ = c2r(H r2c(phi)); v = v_ext(phi~); F_d = c2r(-i k_d H r2c(v))
// therefore collapses to one pass over the half spectrum:
//   F_d(k) = -i k_d H(k)^2 (Q phi(k))/M, with no real-space intermediates.
#include <math.h>
#include <stdint.h>

#include <atomic>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hpf_internal.cuh"

namespace {

constexpr int kThreads = 256;

// Blocks of the readout with the CSVR sums (a grid reduction): two per SM,
// or up to four once each thread would otherwise handle more than three
// beads.  Measured on GB300: 162k beads ran fastest on 304 blocks, 500k
// beads on 608 (1.8 % faster than 304; 1024 blocks was slower than 608).
inline int readout_grid(int64_t n) {
    const int g = reduce_grid(n, kThreads);
    const int64_t per3 = (n + 3 * kThreads - 1) / (3 * kThreads);
    return per3 > g ? (int)std::min<int64_t>(per3, 2 * HPF_REDUCE_GRID) : g;
}

struct TypeScale {
    float s[HPF_MAX_TYPES + 1];
};

struct TypeScaleD {
    double s[HPF_MAX_TYPES + 1];
};

// ---------------------------------------------------------------- paint ---
// One thread per particle; 8 CIC deposits as 64-bit fixed-point integer
// atomics (the weight in units of 2^-24, kFixScale, converted to int32 and
// summed in int64), so the accumulated grid is independent of the
// order in which deposits land: the density is bit-deterministic.
// With `scale` (a barostat's alpha, device double), the positions are first
// rescaled in place, r = float(alpha) * r (hymd/barostat_scr.py:128).
__global__ void k_paint(const float* pos, const int32_t* __restrict__ types,
                        const float* __restrict__ charges, int64_t n, int T,
                        const BoxState* __restrict__ bs, unsigned long long* __restrict__ acc,
                        int64_t M, int* err, const double* __restrict__ scale,
                        const int32_t* __restrict__ idx = nullptr, int64_t n_total = 0) {
    const CicMesh m = cic_mesh(bs);
    const float al = scale ? (float)*scale : 1.0f;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
         j += (int64_t)gridDim.x * blockDim.x) {
        // idx: paint only the listed beads (a compact list of the charged ones)
        const int64_t i = idx ? (int64_t)idx[j] : j;
        if (idx && (i < 0 || i >= n_total)) {
            hpf_flag(err, HPF_ERR_INDEX);
            continue;
        }
        float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        if (scale) {
            x = x * al;
            y = y * al;
            z = z * al;
            float* pw = const_cast<float*>(pos);
            pw[3 * i] = x;
            pw[3 * i + 1] = y;
            pw[3 * i + 2] = z;
        }
        if (!(isfinite(x) && isfinite(y) && isfinite(z))) {
            hpf_flag(err, HPF_ERR_NONFINITE);
            continue;
        }
        int t = 0;
        if (types) {
            t = types[i];
            if (t < 0 || t >= T) {
                hpf_flag(err, HPF_ERR_INDEX);
                continue;
            }
        }
        const float q = charges ? charges[i] : 1.0f;
        if (q == 0.0f) continue;
        cic_deposit(m, x, y, z, q, acc + (int64_t)t * M);
    }
}

// Fixed-point accumulators -> float density (times mass/dV), then clear the
// accumulators for the next paint (so no separate memset is needed).
// Grid: blockIdx.y = grid index g (type), x strides over the mesh.
__global__ void k_paint_finalize(unsigned long long* __restrict__ acc, float* __restrict__ out,
                                 int64_t M, int G, TypeScale sc,
                                 const BoxState* __restrict__ bs) {
    const int g = blockIdx.y;
    const float s = sc.s[g] * bs->inv_dV * kFixInv;
    ulonglong2* a = reinterpret_cast<ulonglong2*>(acc + (int64_t)g * M);
    float4* o4 = reinterpret_cast<float4*>(out + (int64_t)g * M);
    const int64_t M4 = M / 4;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < M4;
         q += (int64_t)gridDim.x * blockDim.x) {
        const ulonglong2 a0 = a[2 * q], a1 = a[2 * q + 1];
        float4 o;
        o.x = fix_to_float((long long)a0.x) * s;
        o.y = fix_to_float((long long)a0.y) * s;
        o.z = fix_to_float((long long)a1.x) * s;
        o.w = fix_to_float((long long)a1.y) * s;
        o4[q] = o;
        a[2 * q] = make_ulonglong2(0ull, 0ull);
        a[2 * q + 1] = make_ulonglong2(0ull, 0ull);
    }
}

// Same for meshes whose size is not a multiple of 4.
__global__ void k_paint_finalize1(unsigned long long* __restrict__ acc, float* __restrict__ out,
                                  int64_t M, int G, TypeScale sc,
                                  const BoxState* __restrict__ bs) {
    const int g = blockIdx.y;
    const float s = sc.s[g] * bs->inv_dV * kFixInv;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < M;
         e += (int64_t)gridDim.x * blockDim.x) {
        out[(int64_t)g * M + e] = fix_to_float((long long)acc[(int64_t)g * M + e]) * s;
        acc[(int64_t)g * M + e] = 0ull;
    }
}

// ---------------------------------------------------------- k-space pass ---
struct KGeom {
    int n0, n1, n2, n2h;
    float invM;
};

__device__ __forceinline__ void mode_k(int64_t idx, const KGeom& g, const BoxState* bs,
                                       float& kx, float& ky, float& kz, float& gx, float& gy,
                                       float& gz, float& wk) {
    const int iz = (int)(idx % g.n2h);
    const int64_t rest = idx / g.n2h;
    const int iy = (int)(rest % g.n1);
    const int ix = (int)(rest / g.n1);
    const int mx = ix <= g.n0 / 2 ? ix : ix - g.n0;
    const int my = iy <= g.n1 / 2 ? iy : iy - g.n1;
    kx = mx * bs->kf[0];
    ky = my * bs->kf[1];
    kz = iz * bs->kf[2];
    // gradient wavevector: the Nyquist index of an even axis carries no
    // odd (derivative) component of a real field
    gx = ((g.n0 & 1) == 0 && ix == g.n0 / 2) ? 0.0f : kx;
    gy = ((g.n1 & 1) == 0 && iy == g.n1 / 2) ? 0.0f : ky;
    gz = ((g.n2 & 1) == 0 && iz == g.n2 / 2) ? 0.0f : kz;
    // half-spectrum multiplicity for Parseval sums
    wk = (iz == 0 || ((g.n2 & 1) == 0 && iz == g.n2 / 2)) ? 1.0f : 2.0f;
}

template <int TT>
__global__ void k_kspace_force(const float2* __restrict__ phi_raw, float2* __restrict__ force_k,
                               float2* __restrict__ phi_f, float2* __restrict__ v_k,
                               int T_rt, int64_t Mc, KGeom g, const BoxState* __restrict__ bs,
                               const Functional* __restrict__ fun, double* sums,
                               double* partials, unsigned int* ticket) {
    constexpr int TM = TT > 0 ? TT : HPF_MAX_TYPES;
    const int T = TT > 0 ? TT : T_rt;
    float Q[TM * TM], bb[TM];
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        bb[i] = i < T ? fun->b[i] : 0.0f;
#pragma unroll
        for (int j = 0; j < TM; ++j) Q[i * TM + j] = (i < T && j < T) ? fun->Q[i * T + j] : 0.0f;
    }
    const float s2h = fun->sigma2_half;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        float kx, ky, kz, gx, gy, gz, wk;
        mode_k(idx, g, bs, kx, ky, kz, gx, gy, gz, wk);
        const float k2 = kx * kx + ky * ky + kz * kz;
        const float H = expf(-s2h * k2);
        const float hm = H * g.invM;
        float2 ph[TM];
#pragma unroll
        for (int j = 0; j < TM; ++j) {
            if (j < T) {
                const float2 r = phi_raw[(int64_t)j * Mc + idx];
                ph[j] = make_float2(r.x * hm, r.y * hm);
                if (phi_f) phi_f[(int64_t)j * Mc + idx] = ph[j];
            } else {
                ph[j] = make_float2(0.0f, 0.0f);
            }
        }
        float q = 0.0f;
#pragma unroll
        for (int t = 0; t < TM; ++t) {
            if (t >= T) break;
            float2 u = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int j = 0; j < TM; ++j) {
                u.x = fmaf(Q[t * TM + j], ph[j].x, u.x);
                u.y = fmaf(Q[t * TM + j], ph[j].y, u.y);
            }
            q = fmaf(ph[t].x, u.x, fmaf(ph[t].y, u.y, q));
            float2 v = make_float2(H * u.x, H * u.y);
            if (idx == 0) v.x += H * bb[t];
            if (v_k) v_k[(int64_t)t * Mc + idx] = v;
            float2* o = force_k + (int64_t)(3 * t) * Mc + idx;
            o[0] = make_float2(gx * v.y, -gx * v.x);
            o[Mc] = make_float2(gy * v.y, -gy * v.x);
            o[2 * Mc] = make_float2(gz * v.y, -gz * v.x);
        }
        if (sums && idx != 0) {
            const float wq = wk * q;
            acc[0] += wq;
            acc[1] = fmaf(wq, kx * kx, acc[1]);
            acc[2] = fmaf(wq, ky * ky, acc[2]);
            acc[3] = fmaf(wq, kz * kz, acc[3]);
        }
    }
    if (sums) grid_reduce_store_f<4, kThreads>(acc, partials, ticket, sums);
}

template <int TT>
__global__ void k_kspace_sums(const float2* __restrict__ phi_f, const float2* __restrict__ psi_k,
                              int T_rt, int64_t Mc, KGeom g, const BoxState* __restrict__ bs,
                              const Functional* __restrict__ fun, TypeScale qt, double* sums,
                              double* partials, unsigned int* ticket) {
    constexpr int TM = TT > 0 ? TT : HPF_MAX_TYPES;
    const int T = TT > 0 ? TT : T_rt;
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        float kx, ky, kz, gx, gy, gz, wk;
        mode_k(idx, g, bs, kx, ky, kz, gx, gy, gz, wk);
        float2 ph[TM];
#pragma unroll
        for (int j = 0; j < TM; ++j)
            ph[j] = j < T ? phi_f[(int64_t)j * Mc + idx] : make_float2(0.0f, 0.0f);
        float q = 0.0f, cr = 0.0f;
        const float2 ps = psi_k ? psi_k[idx] : make_float2(0.0f, 0.0f);
#pragma unroll
        for (int t = 0; t < TM; ++t) {
            if (t >= T) break;
            float2 u = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int j = 0; j < TM; ++j) {
                if (j >= T) break;
                const float Qtj = fun->Q[t * T + j];
                u.x = fmaf(Qtj, ph[j].x, u.x);
                u.y = fmaf(Qtj, ph[j].y, u.y);
            }
            q = fmaf(ph[t].x, u.x, fmaf(ph[t].y, u.y, q));
            cr = fmaf(qt.s[t], fmaf(ps.x, ph[t].x, ps.y * ph[t].y), cr);
        }
        const double kk[3] = {(double)(kx * kx), (double)(ky * ky), (double)(kz * kz)};
        if (idx != 0) {
            const double wq = (double)(wk * q);
            acc[0] += wq;
            for (int d = 0; d < 3; ++d) acc[1 + d] += wq * kk[d];
        }
        const double wc = (double)(wk * cr);
        acc[4] += wc;
        for (int d = 0; d < 3; ++d) acc[5 + d] += wc * kk[d];
    }
    grid_reduce_store<8>(acc, partials, ticket, sums, false);
}

// ---------------------------------------------------------------- readout ---
// Kick fused into the readout (MODE 1), plus CSVR velocity sums (MODE 2).
struct KickDev {
    float* v;
    const float* prev[4];
    int n_prev;
    float mass, h;
    HpfCsvrArgs a;
    const int32_t* group;
    const double* randoms;
    int* counter;
    double* state;
    double* ws;
};

// SCALE: the positions are first multiplied by the isotropic barostat's
// alpha ((float)scale[0], as hpf_scr_scale_positions does) and written back
// through pos_w, which then also serves the reads (pos is not used).
template <int MODE, bool SCALE = false>
__global__ void k_readout(const float* __restrict__ fm, const float* __restrict__ pos,
                          const int32_t* __restrict__ types, const float* __restrict__ charges,
                          int64_t n, int T, int64_t M, const BoxState* __restrict__ bs,
                          float* __restrict__ force, int* err, KickDev kd,
                          const int32_t* __restrict__ idx = nullptr, int64_t n_total = 0,
                          float* pos_w = nullptr, const double* __restrict__ scale = nullptr) {
    pdl_wait();
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int n0 = bs->n[0], n1 = bs->n[1], n2 = bs->n[2];
    const float h0 = bs->ih_hi[0], h1 = bs->ih_hi[1], h2 = bs->ih_hi[2];
    const float l0 = bs->ih_lo[0], l1 = bs->ih_lo[1], l2 = bs->ih_lo[2];
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
         j += (int64_t)gridDim.x * blockDim.x) {
        // idx: read out only the listed beads (MODE 0; the others are untouched)
        const int64_t i = idx ? (int64_t)idx[j] : j;
        if (idx && (i < 0 || i >= n_total)) {
            hpf_flag(err, HPF_ERR_INDEX);
            continue;
        }
        float x, y, z;
        if (SCALE) {
            const float al = (float)scale[0];
            x = pos_w[3 * i] * al;
            y = pos_w[3 * i + 1] * al;
            z = pos_w[3 * i + 2] * al;
            pos_w[3 * i] = x;
            pos_w[3 * i + 1] = y;
            pos_w[3 * i + 2] = z;
        } else {
            x = pos[3 * i];
            y = pos[3 * i + 1];
            z = pos[3 * i + 2];
        }
        float out[3] = {0.0f, 0.0f, 0.0f};
        int t = types ? types[i] : 0;
        const float q = charges ? charges[i] : 1.0f;
        const bool ok = isfinite(x) && isfinite(y) && isfinite(z) && t >= 0 && t < T;
        if (!ok) hpf_flag(err, (t >= 0 && t < T) ? HPF_ERR_NONFINITE : HPF_ERR_INDEX);
        if (ok && q != 0.0f) {
            int ix, iy, iz;
            float fx, fy, fz;
            grid_coord(x, h0, l0, n0, ix, fx);
            grid_coord(y, h1, l1, n1, iy, fy);
            grid_coord(z, h2, l2, n2, iz, fz);
            const int jx = ix + 1 == n0 ? 0 : ix + 1;
            const int jy = iy + 1 == n1 ? 0 : iy + 1;
            const int jz = iz + 1 == n2 ? 0 : iz + 1;
            const float wx[2] = {1.0f - fx, fx}, wy[2] = {1.0f - fy, fy}, wz[2] = {1.0f - fz, fz};
            const int xs[2] = {ix, jx}, ys[2] = {iy, jy}, zs[2] = {iz, jz};
            const float* base = fm + (int64_t)t * 3 * M;
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int b = 0; b < 2; ++b) {
                    const int64_t row = ((int64_t)xs[a] * n1 + ys[b]) * n2;
                    const float wab = wx[a] * wy[b];
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        const float w = wab * wz[c];
                        const int64_t o = row + zs[c];
                        out[0] = fmaf(w, __ldg(base + o), out[0]);
                        out[1] = fmaf(w, __ldg(base + M + o), out[1]);
                        out[2] = fmaf(w, __ldg(base + 2 * M + o), out[2]);
                    }
                }
            out[0] *= q;
            out[1] *= q;
            out[2] *= q;
        }
        force[3 * i] = out[0];
        force[3 * i + 1] = out[1];
        force[3 * i + 2] = out[2];
        if (MODE >= 1) {
            // v += 0.5 dt_o F_q / m for the earlier slow forces, then this one
            float w[3];
            for (int d = 0; d < 3; ++d) {
                float x = kd.v[3 * i + d];
                for (int q2 = 0; q2 < kd.n_prev; ++q2)
                    x = x + kd.h * (kd.prev[q2][3 * i + d] / kd.mass);
                x = x + kd.h * (out[d] / kd.mass);
                kd.v[3 * i + d] = x;
                w[d] = x;
            }
            if (MODE == 2) {
                const int g = kd.group ? kd.group[i] : 0;
                if (g == 0 || g == 1) {
                    acc[4 * g + 0] += w[0];
                    acc[4 * g + 1] += w[1];
                    acc[4 * g + 2] += w[2];
                    acc[4 * g + 3] += fmaf(w[0], w[0], fmaf(w[1], w[1], w[2] * w[2]));
                }
            }
        }
    }
    pdl_trigger();
    if (MODE == 2) {
        if (grid_reduce_store_f<8, kThreads>(acc, ws_partials(kd.ws), ws_ticket(kd.ws), kd.ws))
            csvr_update(kd.a, kd.ws, kd.randoms, kd.counter, kd.state, err);
    }
}

// ------------------------------------------------------------------- PIC ---
__global__ void k_kspace_pic(const float2* __restrict__ rho_raw, float2* __restrict__ out,
                             int64_t Mc, KGeom g, const BoxState* __restrict__ bs,
                             const Functional* __restrict__ fun, float four_pi_fac,
                             double* sums, double* partials, unsigned int* ticket) {
    const float s2h = fun->sigma2_half;
    double acc[1] = {0.0};
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        float kx, ky, kz, gx, gy, gz, wk;
        mode_k(idx, g, bs, kx, ky, kz, gx, gy, gz, wk);
        float k2 = kx * kx + ky * ky + kz * kz;
        const float H = expf(-s2h * k2);
        if (idx == 0) k2 = 1.0f;  // k.normp(p=2, zeromode=1)
        const float2 r = rho_raw[idx];
        const float2 rq = make_float2(r.x * g.invM, r.y * g.invM);  // phi_q(k)
        const float s = four_pi_fac * H / k2;
        const float2 psi = make_float2(rq.x * s, rq.y * s);
        out[idx] = psi;
        out[Mc + idx] = make_float2(gx * psi.y, -gx * psi.x);
        out[2 * Mc + idx] = make_float2(gy * psi.y, -gy * psi.x);
        out[3 * Mc + idx] = make_float2(gz * psi.y, -gz * psi.x);
        if (sums) acc[0] += (double)(wk * fmaf(rq.x, psi.x, rq.y * psi.y));
    }
    if (sums) grid_reduce_store<1>(acc, partials, ticket, sums, false);
}

// ------------------------------------------------------- FP64 energy path ---
// Energies and pressure sums in FP64 from the fixed-point densities: the
// accumulators are converted to double grids, transformed with a D2Z cuFFT
// and reduced over the half spectrum in FP64.  Used where the reference
// reports energies (print steps, barostat), never inside the MD step.
__global__ void k_paint_finalize_f64(unsigned long long* __restrict__ acc,
                                     double* __restrict__ out, int64_t M, int G, TypeScaleD sc,
                                     const BoxState* __restrict__ bs) {
    const double inv_dV = 1.0 / bs->dV;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)G * M;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int g = (int)(e / M);
        out[e] = (double)(long long)acc[e] * (sc.s[g] * inv_dV * (double)kFixInv);
        acc[e] = 0ull;
    }
}

template <int TT>
__global__ void k_energy_f64(const double2* __restrict__ spec, int T_rt, int has_q, int64_t Mc,
                             KGeom g, double invM, const BoxState* __restrict__ bs,
                             const Functional* __restrict__ fun, TypeScale qt, double four_pi_fac,
                             double* out, double* partials, unsigned int* ticket) {
    constexpr int TM = TT > 0 ? TT : HPF_MAX_TYPES;
    const int T = TT > 0 ? TT : T_rt;
    double acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = 0.0;
    const double kf0 = 2.0 * 3.14159265358979323846 / bs->L[0];
    const double kf1 = 2.0 * 3.14159265358979323846 / bs->L[1];
    const double kf2 = 2.0 * 3.14159265358979323846 / bs->L[2];
    const double sig2h = fun->sigma2_half_d;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int iz = (int)(idx % g.n2h);
        const int64_t rest = idx / g.n2h;
        const int iy = (int)(rest % g.n1);
        const int ix = (int)(rest / g.n1);
        const double kx = (ix <= g.n0 / 2 ? ix : ix - g.n0) * kf0;
        const double ky = (iy <= g.n1 / 2 ? iy : iy - g.n1) * kf1;
        const double kz = iz * kf2;
        const double wk = (iz == 0 || ((g.n2 & 1) == 0 && iz == g.n2 / 2)) ? 1.0 : 2.0;
        const double k2 = kx * kx + ky * ky + kz * kz;
        const double H = exp(-sig2h * k2);
        const double kk[3] = {kx * kx, ky * ky, kz * kz};
        double2 ph[TM];
#pragma unroll
        for (int j = 0; j < TM; ++j) {
            if (j < T) {
                const double2 r = spec[(int64_t)j * Mc + idx];
                ph[j] = make_double2(r.x * H * invM, r.y * H * invM);
                if (idx == 0) out[16 + j] = r.x * invM;  // mean of phi_j
            } else {
                ph[j] = make_double2(0.0, 0.0);
            }
        }
        double q = 0.0;
#pragma unroll
        for (int t = 0; t < TM; ++t) {
            if (t >= T) break;
            double ux = 0.0, uy = 0.0;
#pragma unroll
            for (int j = 0; j < TM; ++j) {
                if (j >= T) break;
                const double Qtj = fun->Qd[t * T + j];
                ux += Qtj * ph[j].x;
                uy += Qtj * ph[j].y;
            }
            q += ph[t].x * ux + ph[t].y * uy;
        }
        if (idx != 0) {
            acc[0] += wk * q;
            for (int d = 0; d < 3; ++d) acc[1 + d] += wk * kk[d] * q;
        }
        if (has_q) {
            const double2 r = spec[(int64_t)T * Mc + idx];
            const double2 rho = make_double2(r.x * invM, r.y * invM);
            const double kn = idx == 0 ? 1.0 : k2;  // k.normp(p=2, zeromode=1)
            const double s = four_pi_fac * H / kn;
            const double2 psi = make_double2(rho.x * s, rho.y * s);
            acc[4] += wk * (rho.x * psi.x + rho.y * psi.y);
            double cr = 0.0;
            for (int t = 0; t < T; ++t) cr += (double)qt.s[t] * (psi.x * ph[t].x + psi.y * ph[t].y);
            acc[5] += wk * cr;
            for (int d = 0; d < 3; ++d) acc[6 + d] += wk * kk[d] * cr;
        }
    }
    grid_reduce_store<9>(acc, partials, ticket, out, false);
}

// -------------------------------------------------------------- laplacian ---
// lap[t][d](k) = -k_d^2 phi~_t(k)  (comp_laplacian, hymd/field.py:406-425)
__global__ void k_laplacian(const float2* __restrict__ phi_f, float2* __restrict__ out, int T,
                            int64_t Mc, KGeom g, const BoxState* __restrict__ bs) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        float kx, ky, kz, gx, gy, gz, wk;
        mode_k(idx, g, bs, kx, ky, kz, gx, gy, gz, wk);
        const float kk[3] = {kx * kx, ky * ky, kz * kz};
        for (int t = 0; t < T; ++t) {
            const float2 p = phi_f[(int64_t)t * Mc + idx];
            for (int d = 0; d < 3; ++d)
                out[(int64_t)(3 * t + d) * Mc + idx] = make_float2(-kk[d] * p.x, -kk[d] * p.y);
        }
    }
}

// ---------------------------------------------------------------- adjoint ---
// dW/dx: the filtered potential V_t = H * (Q phi~)_t read out with the
// gradient of the CIC weights (phi_t = m_t/dV sum_i W(g - x_i), so
// dW/dx_i = m_t sum_g V_t(g) grad W(g - x_i)); the constant b_t of
// v_t = (Q phi~ + b)_t drops out of a gradient.
// V_t(k) = H(k)^2 sum_j Q_tj phi_j(k) / M  (phi_j(k): raw r2c spectra).
template <int TT>
__global__ void k_kspace_pot(const float2* __restrict__ phi_raw, float2* __restrict__ out,
                             int T_rt, int64_t Mc, KGeom g, const BoxState* __restrict__ bs,
                             const Functional* __restrict__ fun) {
    constexpr int TM = TT > 0 ? TT : HPF_MAX_TYPES;
    const int T = TT > 0 ? TT : T_rt;
    const float s2h = fun->sigma2_half;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        float kx, ky, kz, gx, gy, gz, wk;
        mode_k(idx, g, bs, kx, ky, kz, gx, gy, gz, wk);
        const float H = expf(-s2h * (kx * kx + ky * ky + kz * kz));
        const float h2m = H * H * g.invM;
        float2 ph[TM];
#pragma unroll
        for (int j = 0; j < TM; ++j)
            ph[j] = j < T ? phi_raw[(int64_t)j * Mc + idx] : make_float2(0.0f, 0.0f);
#pragma unroll
        for (int t = 0; t < TM; ++t) {
            if (t >= T) break;
            float ux = 0.0f, uy = 0.0f;
#pragma unroll
            for (int j = 0; j < TM; ++j) {
                if (j >= T) break;
                const float q = fun->Q[t * T + j];
                ux = fmaf(q, ph[j].x, ux);
                uy = fmaf(q, ph[j].y, uy);
            }
            out[(int64_t)t * Mc + idx] = make_float2(ux * h2m, uy * h2m);
        }
    }
}

__global__ void k_readout_grad(const float* __restrict__ vg, const float* __restrict__ pos,
                               const int32_t* __restrict__ types, int64_t n, int T, int64_t M,
                               const BoxState* __restrict__ bs, TypeScale sc,
                               float* __restrict__ grad, int* err, int accumulate = 0,
                               int per_volume = 0, const float* __restrict__ charges = nullptr) {
    const int n0 = bs->n[0], n1 = bs->n[1], n2 = bs->n[2];
    const float h0 = bs->ih_hi[0], h1 = bs->ih_hi[1], h2 = bs->ih_hi[2];
    const float l0 = bs->ih_lo[0], l1 = bs->ih_lo[1], l2 = bs->ih_lo[2];
    const float i0 = h0 + l0, i1 = h1 + l1, i2 = h2 + l2;  // d(frac)/dx = n/L
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        const int t = types ? types[i] : 0;
        float gr[3] = {0.0f, 0.0f, 0.0f};
        const bool ok = isfinite(x) && isfinite(y) && isfinite(z) && t >= 0 && t < T;
        if (!ok) hpf_flag(err, (t >= 0 && t < T) ? HPF_ERR_NONFINITE : HPF_ERR_INDEX);
        if (ok) {
            int ix, iy, iz;
            float fx, fy, fz;
            grid_coord(x, h0, l0, n0, ix, fx);
            grid_coord(y, h1, l1, n1, iy, fy);
            grid_coord(z, h2, l2, n2, iz, fz);
            const int xs[2] = {ix, ix + 1 == n0 ? 0 : ix + 1};
            const int ys[2] = {iy, iy + 1 == n1 ? 0 : iy + 1};
            const int zs[2] = {iz, iz + 1 == n2 ? 0 : iz + 1};
            const float wx[2] = {1.0f - fx, fx}, wy[2] = {1.0f - fy, fy}, wz[2] = {1.0f - fz, fz};
            const float dx[2] = {-i0, i0}, dy[2] = {-i1, i1}, dz[2] = {-i2, i2};
            const float* base = vg + (int64_t)t * M;
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int b = 0; b < 2; ++b) {
                    const int64_t row = ((int64_t)xs[a] * n1 + ys[b]) * n2;
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        const float v = __ldg(base + row + zs[c]);
                        gr[0] = fmaf(dx[a] * wy[b] * wz[c], v, gr[0]);
                        gr[1] = fmaf(wx[a] * dy[b] * wz[c], v, gr[1]);
                        gr[2] = fmaf(wx[a] * wy[b] * dz[c], v, gr[2]);
                    }
                }
            // charges: the bead's charge in place of its type's scale
            const float w0 = charges ? charges[i] : sc.s[t];
            const float m = per_volume ? w0 * bs->inv_dV : w0;
            gr[0] *= m;
            gr[1] *= m;
            gr[2] *= m;
        }
        if (accumulate) {
            grad[3 * i] += gr[0];
            grad[3 * i + 1] += gr[1];
            grad[3 * i + 2] += gr[2];
        } else {
            grad[3 * i] = gr[0];
            grad[3 * i + 1] = gr[1];
            grad[3 * i + 2] = gr[2];
        }
    }
}

// Parseval sums for the parameter gradients over the raw FP32 spectra of
// the densities (the forward path's r2c): for t <= j,
// s_tj = sum_{k != 0} w_k Re(p_t^* p_j) and
// r = sum_{k != 0} w_k k^2 sum_tj Q_tj Re(p_t^* p_j), p_t = H phi_t(k)/M,
// into out[0..P) (row-major t <= j) and out[P]; out[P+1+t] = mean of phi_t.
// FP32 products, per-thread FP32 sums over a few modes, double-float
// (compensated) block and grid reduction.  With V these give
// sum_g phi~_t phi~_j dV = V (s_tj + mean_t mean_j) and
// sum_tj Q_tj sum_g phi~_j (-lap phi~_t) dV = V r.
template <int TT>
__global__ void k_adjoint_sums(const float2* __restrict__ spec, int64_t Mc, KGeom g,
                               const BoxState* __restrict__ bs,
                               const Functional* __restrict__ fun, double* out, double* partials,
                               unsigned int* ticket) {
    constexpr int P = TT * (TT + 1) / 2;
    float acc[P + 1];
#pragma unroll
    for (int k = 0; k <= P; ++k) acc[k] = 0.0f;
    const float s2h = fun->sigma2_half;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        if (idx == 0) {
#pragma unroll
            for (int j = 0; j < TT; ++j) out[P + 1 + j] = (double)spec[(int64_t)j * Mc].x * g.invM;
            continue;
        }
        float kx, ky, kz, gx, gy, gz, wk;
        mode_k(idx, g, bs, kx, ky, kz, gx, gy, gz, wk);
        const float k2 = kx * kx + ky * ky + kz * kz;
        const float Hm = expf(-s2h * k2) * g.invM;
        float2 ph[TT];
#pragma unroll
        for (int j = 0; j < TT; ++j) {
            const float2 r = spec[(int64_t)j * Mc + idx];
            ph[j] = make_float2(r.x * Hm, r.y * Hm);
        }
        float q = 0.0f;
        int p = 0;
#pragma unroll
        for (int t = 0; t < TT; ++t) {
#pragma unroll
            for (int j = t; j < TT; ++j) {
                const float st = fmaf(ph[t].x, ph[j].x, ph[t].y * ph[j].y);
                acc[p++] += wk * st;
                q = fmaf((j == t ? 1.0f : 2.0f) * fun->Q[t * TT + j], st, q);
            }
        }
        acc[P] = fmaf(wk * k2, q, acc[P]);
    }
    grid_reduce_store_f<P + 1, kThreads>(acc, partials, ticket, out);
}

// ------------------------------------------------------------ host glue ---
int make_plan(hpf_ctx* c, cufftHandle* plan, cufftType type, int batch, size_t* ws) {
    int n[3] = {c->n0, c->n1, c->n2};
    if (cufftCreate(plan) != CUFFT_SUCCESS) return HPF_ERR_CUFFT;
    if (cufftSetAutoAllocation(*plan, 0) != CUFFT_SUCCESS) return HPF_ERR_CUFFT;
    long long idist = type == CUFFT_R2C ? c->M : c->Mc;
    long long odist = type == CUFFT_R2C ? c->Mc : c->M;
    long long nn[3] = {n[0], n[1], n[2]};
    if (cufftMakePlanMany64(*plan, 3, nn, NULL, 1, idist, NULL, 1, odist, type, batch, ws) !=
        CUFFT_SUCCESS)
        return HPF_ERR_CUFFT;
    return HPF_OK;
}

KGeom kgeom(const hpf_ctx* c) {
    KGeom g;
    g.n0 = c->n0;
    g.n1 = c->n1;
    g.n2 = c->n2;
    g.n2h = c->n2 / 2 + 1;
    g.invM = (float)(1.0 / (double)c->M);
    return g;
}

int grid_for(int64_t work, int threads) {
    int64_t b = (work + threads - 1) / threads;
    if (b < 1) b = 1;
    const int64_t cap = 152 * 32;
    return (int)(b < cap ? b : cap);
}

// The FP64 buffers and the D2Z plan (batch T+1: densities + charges) are
// only needed for energies and gradients: created on first use.
int ensure_d2z(hpf_ctx* c) {
    if (c->has_d2z) return HPF_OK;
    const int T = c->T;
    HPF_CUDA_TRY(cudaMalloc(&c->d_grid64, sizeof(double) * (size_t)(T + 1) * c->M));
    HPF_CUDA_TRY(cudaMalloc(&c->d_spec64, sizeof(double2) * (size_t)(T + 1) * c->Mc));
    long long nn[3] = {c->n0, c->n1, c->n2};
    size_t ws = 0;
    if (cufftCreate(&c->plan_d2z) != CUFFT_SUCCESS) return HPF_ERR_CUFFT;
    if (cufftMakePlanMany64(c->plan_d2z, 3, nn, NULL, 1, c->M, NULL, 1, c->Mc, CUFFT_D2Z, T + 1,
                            &ws) != CUFFT_SUCCESS) {
        cufftDestroy(c->plan_d2z);
        return HPF_ERR_CUFFT;
    }
    c->has_d2z = true;
    return HPF_OK;
}

// Densities (fixed-point paint) as FP64 grids and their D2Z spectra in
// d_spec64 (slots 0..T-1; slot T holds the charges when given, else zeros).
int density_spectra_f64(hpf_ctx* c, const float* pos, const int32_t* types, int64_t n,
                        const double* type_mass, const float* charges, cudaStream_t st) {
    int r = ensure_d2z(c);
    if (r != HPF_OK) return r;
    const int T = c->T;
    TypeScaleD sc;
    for (int t = 0; t < T; ++t) sc.s[t] = type_mass[t];
    sc.s[T] = 1.0;
    if (n > 0) {
        k_paint<<<grid_for(n, kThreads), kThreads, 0, st>>>(pos, types, nullptr, n, T, c->d_box,
                                                           c->d_acc, c->M, c->d_err, nullptr);
        HPF_LAUNCH_CHECK();
        if (charges) {
            k_paint<<<grid_for(n, kThreads), kThreads, 0, st>>>(
                pos, nullptr, charges, n, 1, c->d_box, c->d_acc + (int64_t)T * c->M, c->M,
                c->d_err, nullptr);
            HPF_LAUNCH_CHECK();
        }
    }
    k_paint_finalize_f64<<<grid_for((int64_t)(T + 1) * c->M, kThreads), kThreads, 0, st>>>(
        c->d_acc, c->d_grid64, c->M, T + 1, sc, c->d_box);
    HPF_LAUNCH_CHECK();
    if (cufftSetStream(c->plan_d2z, st) != CUFFT_SUCCESS) return HPF_ERR_CUFFT;
    if (cufftExecD2Z(c->plan_d2z, c->d_grid64, reinterpret_cast<cufftDoubleComplex*>(c->d_spec64)) !=
        CUFFT_SUCCESS)
        return HPF_ERR_CUFFT;
    return HPF_OK;
}


int launch_kspace_force(hpf_ctx* c, const float2* phi_raw, float2* force_k, float2* phi_f,
                        float2* v_k, double* sums, cudaStream_t st) {
    KGeom g = kgeom(c);
    const int grid = sums ? reduce_grid(c->Mc, kThreads) : grid_for(c->Mc, kThreads);
    double* part = ws_partials(c->d_ws);
    unsigned int* tick = ws_ticket(c->d_ws);
#define HPF_KSF(TT)                                                                      \
    k_kspace_force<TT><<<grid, kThreads, 0, st>>>(phi_raw, force_k, phi_f, v_k, c->T, c->Mc, \
                                                  g, c->d_box, c->d_fun, sums, part, tick)
    switch (c->T) {
        case 1: HPF_KSF(1); break;
        case 2: HPF_KSF(2); break;
        case 3: HPF_KSF(3); break;
        case 4: HPF_KSF(4); break;
        case 5: HPF_KSF(5); break;
        case 6: HPF_KSF(6); break;
        case 7: HPF_KSF(7); break;
        case 8: HPF_KSF(8); break;
        default: HPF_KSF(0); break;
    }
#undef HPF_KSF
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int do_paint(hpf_ctx* c, const float* pos, const int32_t* types, const float* charges,
             int64_t n, int G, const TypeScale& sc, float* out, cudaStream_t st,
             const double* scale = nullptr, bool finalize = true,
             const int32_t* idx = nullptr, int64_t n_total = 0) {
    // G = number of grids (T for densities; 1 for charges, painted into the
    // accumulator slot after the T density slots); idx: paint only the n
    // listed beads of n_total
    unsigned long long* acc = c->d_acc + (charges ? (int64_t)c->T * c->M : 0);
    if (n > 0) {
        k_paint<<<grid_for(n, kThreads), kThreads, 0, st>>>(pos, types, charges, n,
                                                           charges ? 1 : c->T, c->d_box, acc,
                                                           c->M, c->d_err, scale, idx, n_total);
        HPF_LAUNCH_CHECK();
    }
    if (!finalize) return HPF_OK;  // the fused spectral pass reads the accumulators
    // float4 stores need a 16-byte aligned destination (a caller's view may
    // start at any element)
    if (c->M % 4 == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0) {
        dim3 grid(grid_for(c->M / 4, kThreads), G);
        k_paint_finalize<<<grid, kThreads, 0, st>>>(acc, out, c->M, G, sc, c->d_box);
    } else {
        dim3 grid(grid_for(c->M, kThreads), G);
        k_paint_finalize1<<<grid, kThreads, 0, st>>>(acc, out, c->M, G, sc, c->d_box);
    }
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

// pos_w / scale (both or neither): positions scaled by the barostat's alpha
// and written back in the same pass (k_readout's SCALE).
int launch_readout(hpf_ctx* c, const float* fm, const float* pos, const int32_t* types,
                   const float* charges, int64_t n, int T, float* force, const HpfKick* kick,
                   cudaStream_t st, float* pos_w = nullptr, const double* scale = nullptr) {
    KickDev kd;
    memset(&kd, 0, sizeof(kd));
    int mode = 0;
    if (kick) {
        if (!kick->v || kick->n_prev < 0 || kick->n_prev > 4 || !(kick->mass > 0))
            return HPF_ERR_ARG;
        kd.v = kick->v;
        kd.n_prev = kick->n_prev;
        for (int q = 0; q < kick->n_prev; ++q) {
            if (!kick->prev[q]) return HPF_ERR_ARG;
            kd.prev[q] = kick->prev[q];
        }
        kd.mass = (float)kick->mass;
        kd.h = (float)(0.5 * kick->dt_outer);
        mode = 1;
        if (kick->thermo) {
            const HpfCsvrArgs& a = *kick->thermo;
            if (!kick->randoms || !kick->counter || !kick->state || !kick->ws ||
                a.n_groups < 1 || a.n_groups > 2 || (a.n_groups > 1 && !kick->group))
                return HPF_ERR_ARG;
            kd.a = a;
            kd.group = kick->group;
            kd.randoms = kick->randoms;
            kd.counter = kick->counter;
            kd.state = kick->state;
            kd.ws = kick->ws;
            mode = 2;
        }
    }
    if ((pos_w != nullptr) != (scale != nullptr) || (pos_w && mode == 1)) return HPF_ERR_ARG;
    int* err = mode == 2 && kick->d_err ? kick->d_err : c->d_err;
    const int grid = mode == 2 ? readout_grid(n) : grid_for(n, kThreads);
    const int32_t* no_idx = nullptr;
    const int64_t n_total = 0;
    cudaError_t e;
    if (mode == 0 && pos_w)
        e = launch_pdl(k_readout<0, true>, grid, kThreads, 0, st, fm, pos, types, charges, n, T,
                       c->M, c->d_box, force, err, kd, no_idx, n_total, pos_w, scale);
    else if (mode == 0)
        e = launch_pdl(k_readout<0>, grid, kThreads, 0, st, fm, pos, types, charges, n, T, c->M,
                       c->d_box, force, err, kd, no_idx, n_total, pos_w, scale);
    else if (mode == 1)
        e = launch_pdl(k_readout<1>, grid, kThreads, 0, st, fm, pos, types, charges, n, T, c->M,
                       c->d_box, force, err, kd, no_idx, n_total, pos_w, scale);
    else if (pos_w)
        e = launch_pdl(k_readout<2, true>, grid, kThreads, 0, st, fm, pos, types, charges, n, T,
                       c->M, c->d_box, force, err, kd, no_idx, n_total, pos_w, scale);
    else
        e = launch_pdl(k_readout<2>, grid, kThreads, 0, st, fm, pos, types, charges, n, T, c->M,
                       c->d_box, force, err, kd, no_idx, n_total, pos_w, scale);
    return e == cudaSuccess ? HPF_OK : HPF_ERR_CUDA;
}

SpecBufs main_bufs(hpf_ctx* c) { return SpecBufs{c->d_spec_phi, c->d_spec, c->d_grid, c->d_spec_ws}; }
SpecBufs pic_bufs(hpf_ctx* c) {
    return SpecBufs{c->pic_spec_phi, c->pic_spec, c->pic_grid, c->pic_spec_ws};
}

// The charge chain's scratch, stream and events (first use; refused under
// stream capture, where nothing may be allocated).
int pic_chain_setup(hpf_ctx* c, cudaStream_t st) {
    if (c->pic_stream) return HPF_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
        return HPF_ERR_ARG;
    const size_t words = spectral_ws_words(c);
    if (cudaMalloc(&c->pic_spec_phi, sizeof(float2) * (size_t)c->Mc) != cudaSuccess ||
        cudaMalloc(&c->pic_spec, sizeof(float2) * 2 * (size_t)c->Mc) != cudaSuccess ||
        cudaMalloc(&c->pic_grid, sizeof(float) * 4 * (size_t)c->M) != cudaSuccess ||
        cudaMalloc(&c->pic_spec_ws, sizeof(double) * words) != cudaSuccess ||
        cudaMemset(c->pic_spec_ws, 0, sizeof(double) * words) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->pic_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->pic_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->pic_stream, cudaStreamNonBlocking) != cudaSuccess)
        return HPF_ERR_CUDA;
    return HPF_OK;
}

int exec_r2c(hpf_ctx* c, const float* in, float2* out, int batch, cudaStream_t st) {
    if (batch < 1 || batch > HPF_MAX_TYPES || !c->has_r2c[batch]) return HPF_ERR_ARG;
    cufftHandle p = c->plan_r2c[batch];
    if (cufftSetStream(p, st) != CUFFT_SUCCESS) return HPF_ERR_CUFFT;
    if (cufftExecR2C(p, const_cast<cufftReal*>(in), reinterpret_cast<cufftComplex*>(out)) !=
        CUFFT_SUCCESS)
        return HPF_ERR_CUFFT;
    return HPF_OK;
}

int exec_c2r(hpf_ctx* c, const float2* in, float* out, int batch, cudaStream_t st) {
    if (batch < 1 || batch > 3 * HPF_MAX_TYPES + 1 || !c->has_c2r[batch]) return HPF_ERR_ARG;
    cufftHandle p = c->plan_c2r[batch];
    if (cufftSetStream(p, st) != CUFFT_SUCCESS) return HPF_ERR_CUFFT;
    // cuFFT c2r may overwrite its input; all callers pass scratch spectra.
    if (cufftExecC2R(p, reinterpret_cast<cufftComplex*>(const_cast<float2*>(in)), out) !=
        CUFFT_SUCCESS)
        return HPF_ERR_CUFFT;
    return HPF_OK;
}

}  // namespace

// ================================================================ C ABI ===
extern "C" {

const char* hpf_status_string(int s) {
    switch (s) {
        case HPF_OK: return "HPF_OK";
        case HPF_ERR_ARG: return "HPF_ERR_ARG";
        case HPF_ERR_CUDA: return "HPF_ERR_CUDA";
        case HPF_ERR_CUFFT: return "HPF_ERR_CUFFT";
        case HPF_ERR_INDEX: return "HPF_ERR_INDEX";
        case HPF_ERR_NONFINITE: return "HPF_ERR_NONFINITE";
        case HPF_ERR_TIMEOUT: return "HPF_ERR_TIMEOUT";
        case HPF_ERR_NOT_IMPLEMENTED: return "HPF_ERR_NOT_IMPLEMENTED";
        case HPF_ERR_SCRATCH_LIMIT: return "HPF_ERR_SCRATCH_LIMIT";
        default: return "HPF_ERR_UNKNOWN";
    }
}

int hpf_ctx_destroy(hpf_ctx* c) {
    if (!c) return HPF_OK;
    for (int b = 0; b <= HPF_MAX_TYPES; ++b)
        if (c->has_r2c[b]) cufftDestroy(c->plan_r2c[b]);
    for (int b = 0; b <= 3 * HPF_MAX_TYPES + 1; ++b)
        if (c->has_c2r[b]) cufftDestroy(c->plan_c2r[b]);
    cudaFree(c->fft_work);
    cudaFree(c->d_box);
    cudaFree(c->d_fun);
    cudaFree(c->d_acc);
    cudaFree(c->d_grid);
    cudaFree(c->d_spec);
    cudaFree(c->d_spec_phi);
    cudaFree(c->d_ws);
    cudaFree(c->d_err);
    if (c->has_d2z) cufftDestroy(c->plan_d2z);
    cudaFree(c->d_grid64);
    cudaFree(c->d_spec64);
    cudaFree(c->gpe_grid);
    cudaFree(c->gpe_spec);
    cudaFree(c->gpe_ws);
    cudaFreeHost(c->gpe_host);
    if (c->gpe_exec) cudaGraphExecDestroy(c->gpe_exec);
    if (c->gpe_graph) cudaGraphDestroy(c->gpe_graph);
    if (c->gpe_cap) cudaStreamDestroy(c->gpe_cap);
    cudaFree(c->d_tw);
    cudaFree(c->d_spec_ws);
    cudaFree(c->pic_spec_phi);
    cudaFree(c->pic_spec);
    cudaFree(c->pic_grid);
    cudaFree(c->pic_spec_ws);
    if (c->pic_stream) cudaStreamDestroy(c->pic_stream);
    if (c->pic_fork) cudaEventDestroy(c->pic_fork);
    if (c->pic_join) cudaEventDestroy(c->pic_join);
    free(c);
    return HPF_OK;
}

int hpf_ctx_create(hpf_ctx** out, int n0, int n1, int n2, int T, const double box[3]) {
    if (!out || !box || n0 < 2 || n1 < 2 || n2 < 2 || T < 1 || T > HPF_MAX_TYPES)
        return HPF_ERR_ARG;
    if (!(box[0] > 0 && box[1] > 0 && box[2] > 0)) return HPF_ERR_ARG;
    hpf_ctx* c = (hpf_ctx*)calloc(1, sizeof(hpf_ctx));
    if (!c) return HPF_ERR_ARG;
    c->n0 = n0;
    c->n1 = n1;
    c->n2 = n2;
    c->T = T;
    c->M = (int64_t)n0 * n1 * n2;
    c->Mc = (int64_t)n0 * n1 * (n2 / 2 + 1);
    cudaGetDevice(&c->device);
    const int G = 3 * T > 4 ? 3 * T : 4;
    int st = HPF_OK;
#define CK(x)                      \
    do {                           \
        if ((x) != cudaSuccess) {  \
            st = HPF_ERR_CUDA;     \
            goto fail;             \
        }                          \
    } while (0)
    CK(cudaMalloc(&c->d_box, sizeof(BoxState)));
    CK(cudaMalloc(&c->d_fun, sizeof(Functional)));
    CK(cudaMalloc(&c->d_acc, sizeof(unsigned long long) * (size_t)(T + 1) * c->M));
    CK(cudaMemset(c->d_acc, 0, sizeof(unsigned long long) * (size_t)(T + 1) * c->M));
    CK(cudaMalloc(&c->d_grid, sizeof(float) * (size_t)G * c->M));
    CK(cudaMalloc(&c->d_spec, sizeof(float2) * (size_t)G * c->Mc));
    CK(cudaMalloc(&c->d_spec_phi, sizeof(float2) * (size_t)T * c->Mc));
    CK(cudaMalloc(&c->d_ws, sizeof(double) * HPF_OUT_DOUBLES));
    CK(cudaMemset(c->d_ws, 0, sizeof(double) * HPF_OUT_DOUBLES));
    CK(cudaMalloc(&c->d_err, sizeof(int)));
    CK(cudaMemset(c->d_err, 0, sizeof(int)));
    {
        // plans: r2c for T and 1 grids; c2r for 3T (force mesh), T, 4 (PIC), 1
        size_t need = 0, ws = 0;
        const int r2c_b[2] = {T, 1};
        const int c2r_b[4] = {3 * T, T, 4, 1};
        for (int i = 0; i < 2; ++i) {
            const int b = r2c_b[i];
            if (c->has_r2c[b]) continue;
            if ((st = make_plan(c, &c->plan_r2c[b], CUFFT_R2C, b, &ws)) != HPF_OK) goto fail;
            c->has_r2c[b] = true;
            if (ws > need) need = ws;
        }
        for (int i = 0; i < 4; ++i) {
            const int b = c2r_b[i];
            if (c->has_c2r[b]) continue;
            if ((st = make_plan(c, &c->plan_c2r[b], CUFFT_C2R, b, &ws)) != HPF_OK) goto fail;
            c->has_c2r[b] = true;
            if (ws > need) need = ws;
        }
        c->fft_work_size = need;
        if (need) CK(cudaMalloc(&c->fft_work, need));
        for (int b = 0; b <= HPF_MAX_TYPES; ++b)
            if (c->has_r2c[b] && cufftSetWorkArea(c->plan_r2c[b], c->fft_work) != CUFFT_SUCCESS) {
                st = HPF_ERR_CUFFT;
                goto fail;
            }
        for (int b = 0; b <= 3 * HPF_MAX_TYPES + 1; ++b)
            if (c->has_c2r[b] && cufftSetWorkArea(c->plan_c2r[b], c->fft_work) != CUFFT_SUCCESS) {
                st = HPF_ERR_CUFFT;
                goto fail;
            }
    }
    {
        int nn[3] = {n0, n1, n2};
        fill_box_state(c->h_box, box[0], box[1], box[2], nn);
        CK(cudaMemcpy(c->d_box, &c->h_box, sizeof(BoxState), cudaMemcpyHostToDevice));
        memset(&c->h_fun, 0, sizeof(Functional));
        CK(cudaMemcpy(c->d_fun, &c->h_fun, sizeof(Functional), cudaMemcpyHostToDevice));
    }
#undef CK
    if ((st = spectral_setup(c)) != HPF_OK) goto fail;
    *out = c;
    return HPF_OK;
fail:
    hpf_ctx_destroy(c);
    *out = nullptr;
    return st;
}

int hpf_ctx_set_box(hpf_ctx* c, const double box[3], void* stream) {
    if (!c || !box || !(box[0] > 0 && box[1] > 0 && box[2] > 0)) return HPF_ERR_ARG;
    int nn[3] = {c->n0, c->n1, c->n2};
    fill_box_state(c->h_box, box[0], box[1], box[2], nn);
    HPF_CUDA_TRY(cudaMemcpyAsync(c->d_box, &c->h_box, sizeof(BoxState), cudaMemcpyHostToDevice,
                                 as_stream(stream)));
    HPF_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
    return HPF_OK;
}

int hpf_ctx_set_spectral(hpf_ctx* c, int fused) {
    if (!c || fused < 0 || fused > 1) return HPF_ERR_ARG;
    if (fused && !c->spec_ok) return HPF_ERR_ARG;
    c->spec_fused = fused;
    return HPF_OK;
}

int hpf_ctx_get_spectral(const hpf_ctx* c, int* fused, int* available) {
    if (!c) return HPF_ERR_ARG;
    if (fused) *fused = c->spec_fused;
    if (available) *available = c->spec_ok;
    return HPF_OK;
}

int hpf_ctx_set_spectral_tile(hpf_ctx* c, int width) {
    if (!c) return HPF_ERR_ARG;
    return spectral_set_tile(c, width);
}

int hpf_ctx_get_spectral_tile(const hpf_ctx* c, int* width, int* allowed_mask) {
    if (!c) return HPF_ERR_ARG;
    if (width) *width = c->spec_ok ? c->spec_W : 0;
    if (allowed_mask) {
        int m = 0;
        if (c->spec_ok)
            for (int w = 4; w <= 16; w *= 2)
                if (spectral_tile_ok(c, w)) m |= w;
        *allowed_mask = m;
    }
    return HPF_OK;
}

int hpf_ctx_box_state(hpf_ctx* c, void** d_state) {
    if (!c || !d_state) return HPF_ERR_ARG;
    *d_state = c->d_box;
    return HPF_OK;
}

int hpf_ctx_set_functional(hpf_ctx* c, const double* Q, const double* b, double cc,
                           double sigma) {
    if (!c || !Q || !b) return HPF_ERR_ARG;
    const int T = c->T;
    for (int i = 0; i < T; ++i) {
        c->h_fun.b[i] = (float)b[i];
        c->h_fun.bd[i] = b[i];
        for (int j = 0; j < T; ++j) {
            c->h_fun.Q[i * T + j] = (float)Q[i * T + j];
            c->h_fun.Qd[i * T + j] = Q[i * T + j];
        }
    }
    c->h_fun.c = cc;
    c->h_fun.sigma2_half = (float)(0.5 * sigma * sigma);
    c->h_fun.sigma2_half_d = 0.5 * sigma * sigma;
    HPF_CUDA_TRY(cudaMemcpy(c->d_fun, &c->h_fun, sizeof(Functional), cudaMemcpyHostToDevice));
    return HPF_OK;
}

int hpf_get_error(hpf_ctx* c, void* stream, int* code) {
    if (!c || !code) return HPF_ERR_ARG;
    int h = 0;
    HPF_CUDA_TRY(cudaMemcpyAsync(&h, c->d_err, sizeof(int), cudaMemcpyDeviceToHost,
                                 as_stream(stream)));
    HPF_CUDA_TRY(cudaMemsetAsync(c->d_err, 0, sizeof(int), as_stream(stream)));
    HPF_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
    *code = h;
    return HPF_OK;
}

int hpf_paint(hpf_ctx* c, const float* pos, const int32_t* types, int64_t n,
              const double* type_mass, float* phi_out, void* stream) {
    if (!c || (n > 0 && (!pos || !types)) || !type_mass || !phi_out || n < 0) return HPF_ERR_ARG;
    TypeScale sc;
    for (int t = 0; t < c->T; ++t) sc.s[t] = (float)type_mass[t];
    return do_paint(c, pos, types, nullptr, n, c->T, sc, phi_out, as_stream(stream));
}

int hpf_paint_charge(hpf_ctx* c, const float* pos, const float* charges, int64_t n,
                     float* rho_out, void* stream) {
    if (!c || (n > 0 && (!pos || !charges)) || !rho_out || n < 0) return HPF_ERR_ARG;
    TypeScale sc;
    sc.s[0] = 1.0f;
    return do_paint(c, pos, nullptr, charges, n, 1, sc, rho_out, as_stream(stream));
}

int hpf_r2c(hpf_ctx* c, const float* grids, void* spectra, int batch, void* stream) {
    if (!c || !grids || !spectra) return HPF_ERR_ARG;
    return exec_r2c(c, grids, (float2*)spectra, batch, as_stream(stream));
}

int hpf_c2r(hpf_ctx* c, const void* spectra, float* grids, int batch, void* stream) {
    if (!c || !grids || !spectra) return HPF_ERR_ARG;
    const int G = 3 * c->T > 4 ? 3 * c->T : 4;
    if (batch < 1 || batch > G) return HPF_ERR_ARG;
    // a multi-dimensional cuFFT c2r may overwrite its input; the caller's
    // spectra are preserved by transforming a scratch copy
    cudaStream_t st = as_stream(stream);
    if (spectra != (const void*)c->d_spec)
        HPF_CUDA_TRY(cudaMemcpyAsync(c->d_spec, spectra, sizeof(float2) * batch * c->Mc,
                                     cudaMemcpyDeviceToDevice, st));
    return exec_c2r(c, c->d_spec, grids, batch, st);
}

int hpf_kspace_force(hpf_ctx* c, const void* phi_k_raw, void* force_k, void* phi_fourier,
                     void* v_k, double* sums, void* stream) {
    if (!c || !phi_k_raw || !force_k) return HPF_ERR_ARG;
    return launch_kspace_force(c, (const float2*)phi_k_raw, (float2*)force_k,
                               (float2*)phi_fourier, (float2*)v_k, sums, as_stream(stream));
}

int hpf_kspace_sums(hpf_ctx* c, const void* phi_fourier, const void* psi_k,
                    const double* type_charges, double* sums, void* stream) {
    if (!c || !phi_fourier || !sums) return HPF_ERR_ARG;
    TypeScale qt;
    for (int t = 0; t < c->T; ++t) qt.s[t] = type_charges ? (float)type_charges[t] : 0.0f;
    KGeom g = kgeom(c);
    const int grid = reduce_grid(c->Mc, kThreads);
    cudaStream_t st = as_stream(stream);
    double* part = ws_partials(c->d_ws);
    unsigned int* tick = ws_ticket(c->d_ws);
#define HPF_KSS(TT)                                                                        \
    k_kspace_sums<TT><<<grid, kThreads, 0, st>>>((const float2*)phi_fourier,                 \
                                                 (const float2*)psi_k, c->T, c->Mc, g,      \
                                                 c->d_box, c->d_fun, qt, sums, part, tick)
    switch (c->T) {
        case 1: HPF_KSS(1); break;
        case 2: HPF_KSS(2); break;
        case 3: HPF_KSS(3); break;
        case 4: HPF_KSS(4); break;
        case 5: HPF_KSS(5); break;
        default: HPF_KSS(0); break;
    }
#undef HPF_KSS
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_energy_fp64(hpf_ctx* c, const float* pos, const int32_t* types, int64_t n,
                    const double* type_mass, const float* charges, const double* type_charges,
                    double elec_factor, double* out, void* stream) {
    if (!c || !type_mass || !out || n < 0 || (n > 0 && (!pos || !types))) return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    const int T = c->T;
    int r0 = density_spectra_f64(c, pos, types, n, type_mass, charges, st);
    if (r0 != HPF_OK) return r0;
    TypeScale qt;
    for (int t = 0; t < T; ++t) qt.s[t] = type_charges ? (float)type_charges[t] : 0.0f;
    KGeom g = kgeom(c);
    int grid = reduce_grid(c->Mc, kThreads);
    if (grid > 896) grid = 896;  // 9 partials per block must fit the workspace
    const double fpf = 4.0 * 3.14159265358979323846 * elec_factor;
    double* part = ws_partials(c->d_ws);
    unsigned int* tick = ws_ticket(c->d_ws);
    const int hq = charges ? 1 : 0;
    const double invM = 1.0 / (double)c->M;
#define HPF_KE(TT)                                                                          \
    k_energy_f64<TT><<<grid, kThreads, 0, st>>>(c->d_spec64, T, hq, c->Mc, g, invM, c->d_box, \
                                                c->d_fun, qt, fpf, out, part, tick)
    switch (T) {
        case 1: HPF_KE(1); break;
        case 2: HPF_KE(2); break;
        case 3: HPF_KE(3); break;
        case 4: HPF_KE(4); break;
        case 5: HPF_KE(5); break;
        default: HPF_KE(0); break;
    }
#undef HPF_KE
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_laplacian(hpf_ctx* c, const void* phi_fourier, float* lap_out, void* stream) {
    if (!c || !phi_fourier || !lap_out) return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    k_laplacian<<<grid_for(c->Mc, kThreads), kThreads, 0, st>>>(
        (const float2*)phi_fourier, c->d_spec, c->T, c->Mc, kgeom(c), c->d_box);
    HPF_LAUNCH_CHECK();
    return exec_c2r(c, c->d_spec, lap_out, 3 * c->T, st);
}

int hpf_readout(hpf_ctx* c, const float* force_mesh, const float* pos, const int32_t* types,
                int64_t n, float* force, void* stream) {
    if (!c || !force_mesh || n < 0 || (n > 0 && (!pos || !types || !force))) return HPF_ERR_ARG;
    if (n == 0) return HPF_OK;
    return launch_readout(c, force_mesh, pos, types, nullptr, n, c->T, force, nullptr,
                          as_stream(stream));
}

int hpf_field_step(hpf_ctx* c, float* pos, const int32_t* types, int64_t n,
                   const double* type_mass, float* force, double* sums, const double* pos_scale,
                   const HpfKick* kick, void* stream) {
    if (!c || !type_mass || n < 0 || (n > 0 && (!pos || !types || !force))) return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    TypeScale sc;
    for (int t = 0; t < c->T; ++t) sc.s[t] = (float)type_mass[t];
    int r;
    if (c->spec_fused) {
        if ((r = do_paint(c, pos, types, nullptr, n, c->T, sc, c->d_grid, st, pos_scale,
                          false)) != HPF_OK)
            return r;
        if ((r = spectral_field_force(c, sc.s, sums, st)) != HPF_OK) return r;
        if (n > 0)
            return launch_readout(c, c->d_grid, pos, types, nullptr, n, c->T, force, kick, st);
        return HPF_OK;
    }
    if ((r = do_paint(c, pos, types, nullptr, n, c->T, sc, c->d_grid, st, pos_scale)) != HPF_OK)
        return r;
    if ((r = exec_r2c(c, c->d_grid, c->d_spec_phi, c->T, st)) != HPF_OK) return r;
    if ((r = launch_kspace_force(c, c->d_spec_phi, c->d_spec, nullptr, nullptr, sums, st)) !=
        HPF_OK)
        return r;
    if ((r = exec_c2r(c, c->d_spec, c->d_grid, 3 * c->T, st)) != HPF_OK) return r;
    if (n > 0) return launch_readout(c, c->d_grid, pos, types, nullptr, n, c->T, force, kick, st);
    return HPF_OK;
}

int hpf_field_step_profile(hpf_ctx* c, float* pos, const int32_t* types, int64_t n,
                           const double* type_mass, float* force, double* sums,
                           const double* pos_scale, const HpfKick* kick, void* stream,
                           float* us_out) {
    if (!c || !type_mass || !us_out || n <= 0 || !pos || !types || !force) return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    cudaEvent_t ev[6];
    for (int i = 0; i < 6; ++i) HPF_CUDA_TRY(cudaEventCreate(&ev[i]));
    TypeScale sc;
    for (int t = 0; t < c->T; ++t) sc.s[t] = (float)type_mass[t];
    int r = HPF_OK;
    cudaEventRecord(ev[0], st);
    if (c->spec_fused) {
        // paint (deposits only) | fused passes A+B+C, split evenly | readout:
        // the stage boundaries of the library path are not separate launches
        // here, so "r2c" holds the passes, the next two stages are empty
        if (!r) r = do_paint(c, pos, types, nullptr, n, c->T, sc, c->d_grid, st, pos_scale, false);
        cudaEventRecord(ev[1], st);
        if (!r) r = spectral_field_force(c, sc.s, sums, st);
        cudaEventRecord(ev[2], st);
        cudaEventRecord(ev[3], st);
        cudaEventRecord(ev[4], st);
    } else {
        if (!r) r = do_paint(c, pos, types, nullptr, n, c->T, sc, c->d_grid, st, pos_scale);
        cudaEventRecord(ev[1], st);
        if (!r) r = exec_r2c(c, c->d_grid, c->d_spec_phi, c->T, st);
        cudaEventRecord(ev[2], st);
        if (!r) r = launch_kspace_force(c, c->d_spec_phi, c->d_spec, nullptr, nullptr, sums, st);
        cudaEventRecord(ev[3], st);
        if (!r) r = exec_c2r(c, c->d_spec, c->d_grid, 3 * c->T, st);
        cudaEventRecord(ev[4], st);
    }
    if (!r) r = launch_readout(c, c->d_grid, pos, types, nullptr, n, c->T, force, kick, st);
    cudaEventRecord(ev[5], st);
    cudaEventSynchronize(ev[5]);
    for (int i = 0; i < 5; ++i) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
        us_out[i] = 1000.0f * ms;
    }
    for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
    return r;
}

int hpf_pic_step(hpf_ctx* c, const float* pos, const float* charges, int64_t n,
                 double elec_factor, float* elec_forces, float* phi_q, float* psi,
                 float* elec_field, void* psi_k, double* sums, const HpfKick* kick,
                 void* stream) {
    if (!c || n < 0 || (n > 0 && (!pos || !charges || !elec_forces))) return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    TypeScale sc;
    sc.s[0] = 1.0f;
    const float four_pi_fac = (float)(4.0 * 3.14159265358979323846 * elec_factor);
    int r;
    if (c->spec_fused && !phi_q && !psi_k) {
        // fused passes (no real charge grid or psi spectrum is produced)
        if ((r = do_paint(c, pos, nullptr, charges, n, 1, sc, c->d_grid, st, nullptr, false)) !=
            HPF_OK)
            return r;
        if ((r = spectral_pic(c, main_bufs(c), four_pi_fac, psi != nullptr, sums, st)) != HPF_OK)
            return r;
    } else {
        float* rho = phi_q ? phi_q : c->d_grid;
        if ((r = do_paint(c, pos, nullptr, charges, n, 1, sc, rho, st)) != HPF_OK) return r;
        if ((r = exec_r2c(c, rho, c->d_spec_phi, 1, st)) != HPF_OK) return r;
        KGeom g = kgeom(c);
        const int grid = sums ? reduce_grid(c->Mc, kThreads) : grid_for(c->Mc, kThreads);
        k_kspace_pic<<<grid, kThreads, 0, st>>>(c->d_spec_phi, c->d_spec, c->Mc, g, c->d_box,
                                                c->d_fun, four_pi_fac, sums,
                                                ws_partials(c->d_ws), ws_ticket(c->d_ws));
        HPF_LAUNCH_CHECK();
        if (psi_k)
            HPF_CUDA_TRY(cudaMemcpyAsync(psi_k, c->d_spec, sizeof(float2) * c->Mc,
                                         cudaMemcpyDeviceToDevice, st));
        // c2r of psi and the three field components
        if ((r = exec_c2r(c, c->d_spec, c->d_grid, 4, st)) != HPF_OK) return r;
    }
    if (psi)
        HPF_CUDA_TRY(cudaMemcpyAsync(psi, c->d_grid, sizeof(float) * c->M,
                                     cudaMemcpyDeviceToDevice, st));
    if (elec_field)
        HPF_CUDA_TRY(cudaMemcpyAsync(elec_field, c->d_grid + c->M, sizeof(float) * 3 * c->M,
                                     cudaMemcpyDeviceToDevice, st));
    if (n > 0)
        return launch_readout(c, c->d_grid + c->M, pos, nullptr, charges, n, 1, elec_forces, kick,
                              st);
    return HPF_OK;
}

int hpf_pic_step_list(hpf_ctx* c, const float* pos, const float* charges, const int32_t* idx,
                      int64_t count, int64_t n, double elec_factor, float* elec_forces,
                      double* sums, const HpfKick* kick, void* stream) {
    if (!c || n < 0 || count < 0 || count > n ||
        (count > 0 && (!pos || !charges || !idx || !elec_forces)))
        return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    TypeScale sc;
    sc.s[0] = 1.0f;
    const float four_pi_fac = (float)(4.0 * 3.14159265358979323846 * elec_factor);
    int r;
    if ((r = do_paint(c, pos, nullptr, charges, count, 1, sc, c->d_grid, st, nullptr,
                      !c->spec_fused, idx, n)) != HPF_OK)
        return r;
    if (c->spec_fused) {
        if ((r = spectral_pic(c, main_bufs(c), four_pi_fac, false, sums, st)) != HPF_OK)
            return r;
    } else {
        if ((r = exec_r2c(c, c->d_grid, c->d_spec_phi, 1, st)) != HPF_OK) return r;
        KGeom g = kgeom(c);
        const int kg = sums ? reduce_grid(c->Mc, kThreads) : grid_for(c->Mc, kThreads);
        k_kspace_pic<<<kg, kThreads, 0, st>>>(c->d_spec_phi, c->d_spec, c->Mc, g, c->d_box,
                                              c->d_fun, four_pi_fac, sums, ws_partials(c->d_ws),
                                              ws_ticket(c->d_ws));
        HPF_LAUNCH_CHECK();
        if ((r = exec_c2r(c, c->d_spec, c->d_grid, 4, st)) != HPF_OK) return r;
    }
    // with a kick every bead is visited (the kick and the CSVR sums cover all;
    // the readout gathers only where q != 0), as in hpf_pic_step
    if (kick && n > 0)
        return launch_readout(c, c->d_grid + c->M, pos, nullptr, charges, n, 1, elec_forces, kick,
                              st);
    if (count > 0) {
        KickDev kd;
        memset(&kd, 0, sizeof(kd));
        k_readout<0><<<grid_for(count, kThreads), kThreads, 0, st>>>(
            c->d_grid + c->M, pos, nullptr, charges, count, 1, c->M, c->d_box, elec_forces,
            c->d_err, kd, idx, n);
        HPF_LAUNCH_CHECK();
    }
    return HPF_OK;
}

int hpf_field_pic_step(hpf_ctx* c, float* pos, const int32_t* types, int64_t n,
                       const double* type_mass, float* force, double* sums,
                       const double* pos_scale, const float* charges, const int32_t* idx,
                       int64_t count, double elec_factor, float* elec_forces, double* pic_sums,
                       const HpfKick* kick, int painted, void* stream) {
    if (!c || !type_mass || n < 0 || count < 0 || count > n ||
        (n > 0 && (!pos || !types || !force)) ||
        (count > 0 && (!charges || !idx || !elec_forces)))
        return HPF_ERR_ARG;
    // painted with pos_scale: deposits made at the unscaled positions in the
    // old box (those of the scaled ones in the new box); the density readout
    // scales the positions as it reads them
    float* pos_w = painted && pos_scale ? pos : nullptr;
    const double* rscale = painted ? pos_scale : nullptr;
    cudaStream_t st = as_stream(stream);
    int r;
    if (!c->spec_fused) {
        // the library-FFT path shares its plans' work area: one chain after
        // the other; deposits made elsewhere are not taken
        if (painted) return HPF_ERR_ARG;
        if ((r = hpf_field_step(c, pos, types, n, type_mass, force, sums, pos_scale,
                                charges ? nullptr : kick, stream)) != HPF_OK)
            return r;
        if (!charges) return HPF_OK;
        return hpf_pic_step_list(c, pos, charges, idx, count, n, elec_factor, elec_forces,
                                 pic_sums, kick, stream);
    }
    TypeScale sc, sq;
    for (int t = 0; t < c->T; ++t) sc.s[t] = (float)type_mass[t];
    sq.s[0] = 1.0f;
    if (!charges) {
        // densities only: hpf_field_step, the paint skipped when done already
        if (!painted && (r = do_paint(c, pos, types, nullptr, n, c->T, sc, c->d_grid, st,
                                      pos_scale, false)) != HPF_OK)
            return r;
        if ((r = spectral_field_force(c, sc.s, sums, st)) != HPF_OK) return r;
        if (n > 0)
            return launch_readout(c, c->d_grid, pos, types, nullptr, n, c->T, force, kick, st,
                                  pos_w, rscale);
        return HPF_OK;
    }
    if ((r = pic_chain_setup(c, st)) != HPF_OK) return r;
    const float four_pi_fac = (float)(4.0 * 3.14159265358979323846 * elec_factor);
    // a barostat's rescaling of the positions happens in the density paint:
    // the charge chain starts after it
    if (pos_scale && !painted &&
        (r = do_paint(c, pos, types, nullptr, n, c->T, sc, c->d_grid, st, pos_scale, false)) !=
            HPF_OK)
        return r;
    HPF_CUDA_TRY(cudaEventRecord(c->pic_fork, st));
    HPF_CUDA_TRY(cudaStreamWaitEvent(c->pic_stream, c->pic_fork, 0));
    // charge chain (paint of the listed beads, passes A, B, C) on the second
    // stream; the join below is recorded whatever happened, so that a stream
    // capture is never left forked
    r = painted ? HPF_OK
                : do_paint(c, pos, nullptr, charges, count, 1, sq, c->pic_grid, c->pic_stream,
                           nullptr, false, idx, n);
    if (r == HPF_OK) r = spectral_pic(c, pic_bufs(c), four_pi_fac, false, pic_sums, c->pic_stream);
    const cudaError_t je = cudaEventRecord(c->pic_join, c->pic_stream);
    // density chain on the caller's stream
    int rd = HPF_OK;
    if (!pos_scale && !painted)
        rd = do_paint(c, pos, types, nullptr, n, c->T, sc, c->d_grid, st, nullptr, false);
    if (rd == HPF_OK) rd = spectral_field_force(c, sc.s, sums, st);
    if (rd == HPF_OK && n > 0)
        rd = launch_readout(c, c->d_grid, pos, types, nullptr, n, c->T, force, nullptr, st, pos_w,
                            rscale);
    if (je != cudaSuccess) return HPF_ERR_CUDA;
    HPF_CUDA_TRY(cudaStreamWaitEvent(st, c->pic_join, 0));
    if (r != HPF_OK) return r;
    if (rd != HPF_OK) return rd;
    // charge readout (q E), with the kick and the CSVR sums over every bead
    // when kicking, as hpf_pic_step_list
    if (kick && n > 0)
        return launch_readout(c, c->pic_grid + c->M, pos, nullptr, charges, n, 1, elec_forces,
                              kick, st);
    if (count > 0) {
        KickDev kd;
        memset(&kd, 0, sizeof(kd));
        k_readout<0><<<grid_for(count, kThreads), kThreads, 0, st>>>(
            c->pic_grid + c->M, pos, nullptr, charges, count, 1, c->M, c->d_box, elec_forces,
            c->d_err, kd, idx, n);
        HPF_LAUNCH_CHECK();
    }
    return HPF_OK;
}

}  // extern "C"

// ------------------------------------------------- paint without allocation ---
// Variant of hpf_paint for callers that hold no mesh context and must not
// allocate device memory: the fixed-point accumulators live in one
// file-scope device array, and the box state in the first 256 bytes of it.
// The scratch is shared by every call on a device, so calls that overlap (on
// two streams or two host threads) race.  The first call on a device loads
// the module and looks up the array's address, so it should come before any
// stream capture.  Every call made outside a capture looks the address up
// again (a host-side table lookup once the module is loaded), so a context
// that was destroyed and created again (cudaDeviceReset) is followed; a call
// under capture uses the address of the last call outside one.
namespace {

constexpr int64_t kStaticPaintCells = (int64_t)1 << 21;  // T * n0 * n1 * n2 at most (16 MiB)
constexpr int64_t kStaticBoxBytes = 256;
static_assert(sizeof(BoxState) <= kStaticBoxBytes, "box state exceeds its scratch slot");
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned long long
    g_paint_static_scratch[kStaticBoxBytes / 8 + kStaticPaintCells];

// per device: the array's address from the last lookup outside a capture
std::atomic<char*> g_paint_static_addr[kStaticMaxDevices];

__global__ void k_store_box(BoxState bs, BoxState* dst) { *dst = bs; }

int paint_static_scratch(cudaStream_t st, char** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kStaticMaxDevices)
        return HPF_ERR_CUDA;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) return HPF_ERR_CUDA;
    if (cap == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_paint_static_scratch) != cudaSuccess || !p)
            return HPF_ERR_CUDA;
        g_paint_static_addr[dev].store(static_cast<char*>(p), std::memory_order_release);
    }
    char* p = g_paint_static_addr[dev].load(std::memory_order_acquire);
    if (!p) return HPF_ERR_ARG;  // first call on this device made under capture
    *out = p;
    return HPF_OK;
}

}  // namespace

extern "C" int hpf_paint_static(const float* pos, const int32_t* types, int64_t n, int T, int n0,
                                int n1, int n2, const double box[3], const double* type_mass,
                                float* phi_out, int* d_err, void* stream) {
    if ((n > 0 && (!pos || !types)) || n < 0 || !box || !type_mass || !phi_out || T < 1 ||
        T > HPF_MAX_TYPES || n0 < 2 || n1 < 2 || n2 < 2)
        return HPF_ERR_ARG;
    if (!(box[0] > 0 && box[1] > 0 && box[2] > 0)) return HPF_ERR_ARG;
    const int64_t M = (int64_t)n0 * n1 * n2;
    if (M > kStaticPaintCells || (int64_t)T * M > kStaticPaintCells) return HPF_ERR_SCRATCH_LIMIT;
    cudaStream_t st = as_stream(stream);
    char* base = nullptr;
    int r = paint_static_scratch(st, &base);
    if (r != HPF_OK) return r;
    BoxState* bs = reinterpret_cast<BoxState*>(base);
    unsigned long long* acc = reinterpret_cast<unsigned long long*>(base + kStaticBoxBytes);
    BoxState h;
    memset(&h, 0, sizeof(h));
    const int nn[3] = {n0, n1, n2};
    fill_box_state(h, box[0], box[1], box[2], nn);
    k_store_box<<<1, 1, 0, st>>>(h, bs);
    HPF_LAUNCH_CHECK();
    // the accumulators must start at zero
    HPF_CUDA_TRY(cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * (size_t)T * M, st));
    TypeScale sc;
    for (int t = 0; t < T; ++t) sc.s[t] = (float)type_mass[t];
    if (n > 0) {
        k_paint<<<grid_for(n, kThreads), kThreads, 0, st>>>(pos, types, nullptr, n, T, bs, acc, M,
                                                           d_err, nullptr);
        HPF_LAUNCH_CHECK();
    }
    if (M % 4 == 0 && (reinterpret_cast<uintptr_t>(phi_out) & 15) == 0) {
        dim3 grid(grid_for(M / 4, kThreads), T);
        k_paint_finalize<<<grid, kThreads, 0, st>>>(acc, phi_out, M, T, sc, bs);
    } else {
        dim3 grid(grid_for(M, kThreads), T);
        k_paint_finalize1<<<grid, kThreads, 0, st>>>(acc, phi_out, M, T, sc, bs);
    }
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

// ---------------------------------------------------------------- adjoint ---
extern "C" int hpf_field_adjoint(hpf_ctx* c, const float* pos, const int32_t* types, int64_t n,
                                 const double* type_mass, float* grad_pos, double* sums,
                                 void* stream) {
    if (!c || !type_mass || n < 0 || (n > 0 && (!pos || !types)) || (!grad_pos && !sums))
        return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    const int T = c->T;
    if (sums && T > 8) return HPF_ERR_NOT_IMPLEMENTED;
    int r;
    // densities and their raw spectra, shared by both parts
    TypeScale sc;
    for (int t = 0; t < T; ++t) sc.s[t] = (float)type_mass[t];
    if ((r = do_paint(c, pos, types, nullptr, n, T, sc, c->d_grid, st)) != HPF_OK) return r;
    if ((r = exec_r2c(c, c->d_grid, c->d_spec_phi, T, st)) != HPF_OK) return r;
    if (grad_pos && n > 0) {
        const KGeom g = kgeom(c);
        const int grid = grid_for(c->Mc, kThreads);
#define HPF_KP(TT)                                                                       \
    k_kspace_pot<TT><<<grid, kThreads, 0, st>>>(c->d_spec_phi, c->d_spec, T, c->Mc, g, c->d_box, \
                                                c->d_fun)
        switch (T) {
            case 1: HPF_KP(1); break;
            case 2: HPF_KP(2); break;
            case 3: HPF_KP(3); break;
            case 4: HPF_KP(4); break;
            case 5: HPF_KP(5); break;
            case 6: HPF_KP(6); break;
            case 7: HPF_KP(7); break;
            case 8: HPF_KP(8); break;
            default: HPF_KP(0); break;
        }
#undef HPF_KP
        HPF_LAUNCH_CHECK();
        if ((r = exec_c2r(c, c->d_spec, c->d_grid, T, st)) != HPF_OK) return r;
        k_readout_grad<<<grid_for(n, kThreads), kThreads, 0, st>>>(c->d_grid, pos, types, n, T,
                                                                   c->M, c->d_box, sc, grad_pos,
                                                                   c->d_err);
        HPF_LAUNCH_CHECK();
    }
    if (sums) {
        const KGeom g = kgeom(c);
        const int K = T * (T + 1) / 2 + 1;
        int grid = reduce_grid(c->Mc, kThreads);
        // K partials (float2) per block must fit the workspace's 8 * HPF_REDUCE_BLOCKS slots
        if (grid > 8 * HPF_REDUCE_BLOCKS / K) grid = 8 * HPF_REDUCE_BLOCKS / K;
        double* part = ws_partials(c->d_ws);
        unsigned int* tick = ws_ticket(c->d_ws);
#define HPF_KA(TT)                                                                          \
    k_adjoint_sums<TT><<<grid, kThreads, 0, st>>>(c->d_spec_phi, c->Mc, g, c->d_box, c->d_fun, \
                                                  sums, part, tick)
        switch (T) {
            case 1: HPF_KA(1); break;
            case 2: HPF_KA(2); break;
            case 3: HPF_KA(3); break;
            case 4: HPF_KA(4); break;
            case 5: HPF_KA(5); break;
            case 6: HPF_KA(6); break;
            case 7: HPF_KA(7); break;
            default: HPF_KA(8); break;
        }
#undef HPF_KA
        HPF_LAUNCH_CHECK();
    }
    return HPF_OK;
}

// ------------------------------------------------------ PIC_Spectral_GPE ---
// Electrostatics with a density-weighted dielectric (hymd/field.py:764-1112):
// eps(r) = sum_t eps_t phi~_t / sum_t phi~_t, the generalised Poisson
// equation div(eps grad psi) = -rho~ solved by the reference's polarisation
// iteration, then forces from V_t = q_t psi - (eps_t - eps) |E|^2 / (2 eps0^-1
// sum phi~).  All transforms and products follow the reference's sequence;
// its masked divisions (np.divide(..., where=...)) keep the previous values
// where the mask is false, so phi_eps, the polarisation and |E|^2 / sum phi~
// live in caller-owned grids across calls.
namespace {

enum { kGpeQ = 0, kGpeTot = 1, kGpeEta = 2, kGpeX = 5, kGpeE = 6, kGpePsi = 9, kGpeGrids = 10 };

// spec *= H(k) / M (filter under the unnormalised r2c)
__global__ void k_gpe_filter(float2* __restrict__ spec, int64_t Mc, KGeom g,
                             const BoxState* __restrict__ bs, const Functional* __restrict__ fun) {
    const float s2h = fun->sigma2_half;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        float kx, ky, kz, gx, gy, gz, wk;
        mode_k(idx, g, bs, kx, ky, kz, gx, gy, gz, wk);
        const float s = expf(-s2h * (kx * kx + ky * ky + kz * kz)) * g.invM;
        const float2 v = spec[idx];
        spec[idx] = make_float2(v.x * s, v.y * s);
    }
}

// total density, dielectric (kept where the total is <= 1e-6), q = rho~/eps
// (rho~ kept where eps <= 1e-6) and the first iteration's X = q + pol_prev
__global__ void k_gpe_eps(const float* __restrict__ phi, int T, int64_t M, TypeScale eps_t,
                          float* __restrict__ rho_q, float* __restrict__ tot,
                          float* __restrict__ phi_eps, const float* __restrict__ pol_prev,
                          float* __restrict__ X) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < M;
         e += (int64_t)gridDim.x * blockDim.x) {
        float ts = 0.0f, num = 0.0f;
        for (int t = 0; t < T; ++t) {
            const float p = phi[(int64_t)t * M + e];
            ts = ts + p;
            num = num + eps_t.s[t] * p;
        }
        float pe = phi_eps[e];
        if (ts > 1e-6f) {
            pe = num / ts;
            phi_eps[e] = pe;
        }
        tot[e] = ts;
        const float r = rho_q[e];
        const float q = pe > 1e-6f ? r / pe : r;
        rho_q[e] = q;
        X[e] = q + pol_prev[e];
    }
}

// out[d] = sign * i k'_d in / M (k' the gradient wavevector)
__global__ void k_gpe_grad_spec(const float2* __restrict__ in, float2* __restrict__ out,
                                int64_t Mc, KGeom g, const BoxState* __restrict__ bs,
                                float sign) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        float kx, ky, kz, gx, gy, gz, wk;
        mode_k(idx, g, bs, kx, ky, kz, gx, gy, gz, wk);
        const float2 v = in[idx];
        const float gk[3] = {gx, gy, gz};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float k = sign * gk[d] * g.invM;
            out[(int64_t)d * Mc + idx] = make_float2(-k * v.y, k * v.x);
        }
    }
}

// v = scale in / (M knorm); psi_k = v (when given); out[d] = -i k'_d v
__global__ void k_gpe_field_spec(const float2* __restrict__ in, float2* __restrict__ out,
                                 float2* __restrict__ psi_k, int64_t Mc, KGeom g,
                                 const BoxState* __restrict__ bs, float scale) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        float kx, ky, kz, gx, gy, gz, wk;
        mode_k(idx, g, bs, kx, ky, kz, gx, gy, gz, wk);
        const float k2 = kx * kx + ky * ky + kz * kz;
        const float s = scale * g.invM / (idx == 0 ? 1.0f : k2);
        const float2 v = make_float2(in[idx].x * s, in[idx].y * s);
        if (psi_k) psi_k[idx] = v;
        const float gk[3] = {gx, gy, gz};
#pragma unroll
        for (int d = 0; d < 3; ++d)
            out[(int64_t)d * Mc + idx] = make_float2(gk[d] * v.y, -gk[d] * v.x);
    }
}

__global__ void k_gpe_eta_div(float* __restrict__ eta, const float* __restrict__ phi_eps,
                              int64_t M) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < M;
         e += (int64_t)gridDim.x * blockDim.x) {
        const float pe = phi_eps[e];
        if (pe > 1e-6f)
            for (int d = 0; d < 3; ++d) eta[(int64_t)d * M + e] /= pe;
    }
}

// one polarisation update: pol = w (-eta.E) + (1 - w) pol_prev, the
// convergence measure of |pol - pol_prev| (KIND 0 max, 1 sum, 2 sum of
// squares), pol_prev = pol, X = q + pol
template <int KIND>
__global__ void k_gpe_pol(const float* __restrict__ eta, const float* __restrict__ E,
                          const float* __restrict__ q, float* __restrict__ pol,
                          float* __restrict__ X, int64_t M, float w,
                          unsigned int* __restrict__ max_bits, double* ws) {
    float loc = 0.0f;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < M;
         e += (int64_t)gridDim.x * blockDim.x) {
        const float p0 = -(eta[e] * E[e] + eta[M + e] * E[M + e] + eta[2 * M + e] * E[2 * M + e]);
        const float pp = pol[e];
        const float p = w * p0 + (1.0f - w) * pp;
        const float d = fabsf(p - pp);
        if (KIND == 0) loc = fmaxf(loc, d);
        else if (KIND == 1) loc += d;
        else loc = fmaf(d, d, loc);
        pol[e] = p;
        X[e] = q[e] + p;
    }
    if (KIND == 0) {
        // max is order-independent: atomics on the bit pattern of non-negative floats
        for (int o = 16; o > 0; o >>= 1) loc = fmaxf(loc, __shfl_down_sync(0xffffffffu, loc, o));
        if ((threadIdx.x & 31) == 0) atomicMax(max_bits, __float_as_uint(loc));
    } else {
        float acc[1] = {loc};
        grid_reduce_store_f<1, kThreads>(acc, ws_partials(ws), ws_ticket(ws), ws);
    }
}

// |E|^2, the kept |E|^2 / sum phi~, the external potentials V_t and the
// energy sum of phi_eps |E|^2 (energy = scale * sum)
__global__ void k_gpe_vbar(const float* __restrict__ E, const float* __restrict__ psi,
                           const float* __restrict__ tot, const float* __restrict__ phi_eps,
                           float* __restrict__ contrib, int T, int64_t M, TypeScale eps_t,
                           TypeScale q_t, float half_e0, float* __restrict__ vbar,
                           float* __restrict__ dot_out, double* ws, double* energy,
                           const BoxState* __restrict__ bs, double half_e0_d) {
    float acc[1] = {0.0f};
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < M;
         e += (int64_t)gridDim.x * blockDim.x) {
        const float d = E[e] * E[e] + E[M + e] * E[M + e] + E[2 * M + e] * E[2 * M + e];
        if (tot[e] > 1e-6f) contrib[e] = d / tot[e];
        const float c = contrib[e], pe = phi_eps[e], ps = psi[e];
        for (int t = 0; t < T; ++t)
            vbar[(int64_t)t * M + e] = q_t.s[t] * ps - half_e0 * (eps_t.s[t] - pe) * c;
        if (dot_out) dot_out[e] = d;
        acc[0] = fmaf(pe, d, acc[0]);
    }
    if (grid_reduce_store_f<1, kThreads>(acc, ws_partials(ws), ws_ticket(ws), ws) && energy)
        *energy = bs->dV * half_e0_d * ws[0];  // the current (device) box
}

// F_t,d(k) = -i k'_d H(k) V_t(k) / M
__global__ void k_gpe_force_spec(const float2* __restrict__ vk, float2* __restrict__ out, int T,
                                 int64_t Mc, KGeom g, const BoxState* __restrict__ bs,
                                 const Functional* __restrict__ fun) {
    const float s2h = fun->sigma2_half;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        float kx, ky, kz, gx, gy, gz, wk;
        mode_k(idx, g, bs, kx, ky, kz, gx, gy, gz, wk);
        const float s = expf(-s2h * (kx * kx + ky * ky + kz * kz)) * g.invM;
        const float gk[3] = {gx, gy, gz};
        for (int t = 0; t < T; ++t) {
            const float2 v = vk[(int64_t)t * Mc + idx];
            const float2 h = make_float2(v.x * s, v.y * s);
#pragma unroll
            for (int d = 0; d < 3; ++d)
                out[(int64_t)(3 * t + d) * Mc + idx] = make_float2(gk[d] * h.y, -gk[d] * h.x);
        }
    }
}

// The polarisation loop's device state: the iteration counter and the max
// measure's bits in the tail of gpe_ws.
unsigned int* gpe_max_bits(hpf_ctx* c) {
    return reinterpret_cast<unsigned int*>(c->gpe_ws + 8 + 8 * HPF_REDUCE_BLOCKS + 2);
}
int* gpe_iter(hpf_ctx* c) {
    return reinterpret_cast<int*>(c->gpe_ws + 8 + 8 * HPF_REDUCE_BLOCKS + 3);
}

// before the loop: counter and max measure cleared; the loop runs when the
// reference's `while it < max_iter and delta > conv_crit` holds for it = 0,
// delta = 1
__global__ void k_gpe_loop_init(int* it, unsigned int* max_bits, cudaGraphConditionalHandle h,
                                int run) {
    *it = 0;
    *max_bits = 0u;
    cudaGraphSetConditional(h, run ? 1u : 0u);
}

// after each update: the measure (KIND 0 max from its bits, else the grid
// sum), one more iteration counted, and the loop test for the next
template <int KIND>
__global__ void k_gpe_loop_test(int* it, unsigned int* max_bits, const double* ws,
                                cudaGraphConditionalHandle h, int max_iter, double crit) {
    double delta;
    if (KIND == 0) {
        delta = (double)__uint_as_float(*max_bits);
        *max_bits = 0u;
    } else {
        delta = ws[0];
    }
    const int n = *it + 1;
    *it = n;
    cudaGraphSetConditional(h, (n < max_iter && delta > crit) ? 1u : 0u);
}

int gpe_scratch(hpf_ctx* c) {
    if (c->gpe_grid) return HPF_OK;
    HPF_CUDA_TRY(cudaMalloc(&c->gpe_grid, sizeof(float) * (size_t)kGpeGrids * c->M));
    HPF_CUDA_TRY(cudaMalloc(&c->gpe_spec, sizeof(float2) * (size_t)4 * c->Mc));
    HPF_CUDA_TRY(cudaMalloc(&c->gpe_ws, sizeof(double) * HPF_OUT_DOUBLES));
    HPF_CUDA_TRY(cudaMemset(c->gpe_ws, 0, sizeof(double) * HPF_OUT_DOUBLES));
    HPF_CUDA_TRY(cudaMallocHost(&c->gpe_host, sizeof(double) * 2));
    return HPF_OK;
}

// psi = scale c2r(r2c(X) / (M k^2)) into *psi_grid (when psi_grid is given)
// and E_d = c2r(-i k'_d ...) into the E grids: the fused spectral passes of
// the PIC chain on the real grid X without the filter (psi then lands in
// X's slot, after pass A has read X), or cuFFT with k_gpe_field_spec.
int gpe_field(hpf_ctx* c, float scale, float** psi_grid, cudaStream_t st) {
    const int64_t M = c->M, Mc = c->Mc;
    float* G = c->gpe_grid;
    float2* S = c->gpe_spec;
    int r;
    if (c->spec_fused) {
        const SpecBufs b{S, S + Mc, G + (kGpeE - 1) * M, c->d_spec_ws};
        static_assert(kGpeE - 1 == kGpeX, "psi takes X's slot");
        if ((r = spectral_pic(c, b, scale, psi_grid != nullptr, nullptr, st, G + kGpeX * M,
                              false)) != HPF_OK)
            return r;
        if (psi_grid) *psi_grid = G + kGpeX * M;
        return HPF_OK;
    }
    const KGeom g = kgeom(c);
    const int gk = grid_for(Mc, kThreads);
    if ((r = exec_r2c(c, G + kGpeX * M, S, 1, st)) != HPF_OK) return r;
    k_gpe_field_spec<<<gk, kThreads, 0, st>>>(S, S + Mc, psi_grid ? S : nullptr, Mc, g, c->d_box,
                                              scale);
    HPF_LAUNCH_CHECK();
    for (int d = 0; d < 3; ++d)
        if ((r = exec_c2r(c, S + (1 + d) * Mc, G + (kGpeE + d) * M, 1, st)) != HPF_OK) return r;
    if (psi_grid) {
        if ((r = exec_c2r(c, S, G + kGpePsi * M, 1, st)) != HPF_OK) return r;
        *psi_grid = G + kGpePsi * M;
    }
    return HPF_OK;
}

// One polarisation update on `st`: X -> E (3 grids), then pol and X updated
// and the measure taken.
int gpe_update(hpf_ctx* c, float* pol, int kind, float w, cudaStream_t st) {
    const int64_t M = c->M;
    float* G = c->gpe_grid;
    const int rg = reduce_grid(M, kThreads);
    int r;
    if ((r = gpe_field(c, 1.0f, nullptr, st)) != HPF_OK) return r;
    unsigned int* mb = gpe_max_bits(c);
    if (kind == 0)
        k_gpe_pol<0><<<rg, kThreads, 0, st>>>(G + kGpeEta * M, G + kGpeE * M, G + kGpeQ * M, pol,
                                              G + kGpeX * M, M, w, mb, c->gpe_ws);
    else if (kind == 1)
        k_gpe_pol<1><<<rg, kThreads, 0, st>>>(G + kGpeEta * M, G + kGpeE * M, G + kGpeQ * M, pol,
                                              G + kGpeX * M, M, w, mb, c->gpe_ws);
    else
        k_gpe_pol<2><<<rg, kThreads, 0, st>>>(G + kGpeEta * M, G + kGpeE * M, G + kGpeQ * M, pol,
                                              G + kGpeX * M, M, w, mb, c->gpe_ws);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

// The loop graph: init kernel -> while node { update, test }, captured on the
// context's own stream (cuFFT included) and instantiated once per parameter
// set.  The handle's launch default is 0, so a graph whose init kernel did
// not run executes no iteration.
int gpe_loop_graph(hpf_ctx* c, float* pol, int kind, double mixing, double crit, int max_iter) {
    if (c->gpe_exec && c->gpe_key_pol == pol && c->gpe_key_kind == kind &&
        c->gpe_key_mix == mixing && c->gpe_key_crit == crit && c->gpe_key_max == max_iter)
        return HPF_OK;
    if (c->gpe_exec) cudaGraphExecDestroy(c->gpe_exec);
    if (c->gpe_graph) cudaGraphDestroy(c->gpe_graph);
    c->gpe_exec = nullptr;
    c->gpe_graph = nullptr;
    if (!c->gpe_cap) HPF_CUDA_TRY(cudaStreamCreateWithFlags(&c->gpe_cap, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    HPF_CUDA_TRY(cudaGraphCreate(&g, 0));
    c->gpe_graph = g;
    cudaGraphConditionalHandle h;
    HPF_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
    cudaStream_t cs = c->gpe_cap;
    int* it = gpe_iter(c);
    unsigned int* mb = gpe_max_bits(c);
    HPF_CUDA_TRY(cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal));
    k_gpe_loop_init<<<1, 1, 0, cs>>>(it, mb, h, max_iter > 0 && 1.0 > crit);
    cudaGraph_t g2 = nullptr;
    const cudaError_t e1 = cudaGetLastError();
    HPF_CUDA_TRY(cudaStreamEndCapture(cs, &g2));
    if (e1 != cudaSuccess) return HPF_ERR_CUDA;
    cudaGraphNode_t init = nullptr;
    size_t count = 1;
    HPF_CUDA_TRY(cudaGraphGetNodes(g, &init, &count));
    if (count != 1) return HPF_ERR_CUDA;
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t loop = nullptr;
    HPF_CUDA_TRY(cudaGraphAddNode(&loop, g, &init, nullptr, 1, &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    HPF_CUDA_TRY(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal));
    int r = gpe_update(c, pol, kind, (float)mixing, cs);
    if (r == HPF_OK) {
        if (kind == 0)
            k_gpe_loop_test<0><<<1, 1, 0, cs>>>(it, mb, c->gpe_ws, h, max_iter, crit);
        else
            k_gpe_loop_test<1><<<1, 1, 0, cs>>>(it, mb, c->gpe_ws, h, max_iter, crit);
        if (cudaGetLastError() != cudaSuccess) r = HPF_ERR_CUDA;
    }
    cudaGraph_t b2 = nullptr;
    HPF_CUDA_TRY(cudaStreamEndCapture(cs, &b2));
    if (r != HPF_OK) return r;
    HPF_CUDA_TRY(cudaGraphInstantiate(&c->gpe_exec, g, 0));
    c->gpe_key_pol = pol;
    c->gpe_key_kind = kind;
    c->gpe_key_mix = mixing;
    c->gpe_key_crit = crit;
    c->gpe_key_max = max_iter;
    return HPF_OK;
}

}  // namespace

extern "C" int hpf_gpe_step(hpf_ctx* c, const float* pos, const int32_t* types,
                            const float* charges, int64_t n, const float* phi_tilde,
                            const double* eps_type, const double* type_charges,
                            double coulomb_constant, double conv_crit, double mixing,
                            int conv_kind, int max_iter, float* phi_eps, float* pol_prev,
                            float* contrib, float* elec_forces, float* psi_out,
                            float* elec_field_out, float* elec_dot_out, float* vbar_out,
                            double* energy_out, int* iterations, void* stream) {
    if (!c || n < 0 || (n > 0 && (!pos || !types || !charges || !elec_forces)) || !phi_tilde ||
        !eps_type || !type_charges || !phi_eps || !pol_prev || !contrib || conv_kind < 0 ||
        conv_kind > 2 || max_iter < 0 || !(coulomb_constant > 0))
        return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
        return HPF_ERR_ARG;
    int r = gpe_scratch(c);
    if (r != HPF_OK) return r;
    const int T = c->T;
    const int64_t M = c->M, Mc = c->Mc;
    float* G = c->gpe_grid;
    float2* S = c->gpe_spec;  // [0] scalar spectrum, [1..3] vector spectra
    const KGeom g = kgeom(c);
    const int gm = grid_for(M, kThreads), gk = grid_for(Mc, kThreads);
    TypeScale eps_t, q_t, one;
    for (int t = 0; t < T; ++t) {
        eps_t.s[t] = (float)eps_type[t];
        q_t.s[t] = (float)type_charges[t];
    }
    one.s[0] = 1.0f;
    // filtered charge density rho~ = c2r(H r2c(q / dV))
    if ((r = do_paint(c, pos, nullptr, charges, n, 1, one, G + kGpeQ * M, st)) != HPF_OK) return r;
    if ((r = exec_r2c(c, G + kGpeQ * M, S, 1, st)) != HPF_OK) return r;
    k_gpe_filter<<<gk, kThreads, 0, st>>>(S, Mc, g, c->d_box, c->d_fun);
    HPF_LAUNCH_CHECK();
    if ((r = exec_c2r(c, S, G + kGpeQ * M, 1, st)) != HPF_OK) return r;
    // dielectric, q = rho~/eps, X = q + pol_prev
    k_gpe_eps<<<gm, kThreads, 0, st>>>(phi_tilde, T, M, eps_t, G + kGpeQ * M, G + kGpeTot * M,
                                       phi_eps, pol_prev, G + kGpeX * M);
    HPF_LAUNCH_CHECK();
    // eta_d = (i k_d eps)(r) / eps
    if ((r = exec_r2c(c, phi_eps, S, 1, st)) != HPF_OK) return r;
    k_gpe_grad_spec<<<gk, kThreads, 0, st>>>(S, S + Mc, Mc, g, c->d_box, 1.0f);
    HPF_LAUNCH_CHECK();
    for (int d = 0; d < 3; ++d)
        if ((r = exec_c2r(c, S + (1 + d) * Mc, G + (kGpeEta + d) * M, 1, st)) != HPF_OK) return r;
    k_gpe_eta_div<<<gm, kThreads, 0, st>>>(G + kGpeEta * M, phi_eps, M);
    HPF_LAUNCH_CHECK();
    // polarisation iteration: the reference tests convergence after every
    // update; here the test runs on the device and drives the while node of
    // the loop graph, so the loop needs no host round trip
    if ((r = gpe_loop_graph(c, pol_prev, conv_kind, mixing, conv_crit, max_iter)) != HPF_OK)
        return r;
    HPF_CUDA_TRY(cudaGraphLaunch(c->gpe_exec, st));
    const int rg = reduce_grid(M, kThreads);
    // psi = c2r(eps0^-1 r2c(q + pol) / k^2), E = c2r(-i k psi_k)
    const double e0inv = coulomb_constant * 4.0 * 3.14159265358979323846;
    float* psi_grid = nullptr;
    if ((r = gpe_field(c, (float)e0inv, &psi_grid, st)) != HPF_OK) return r;
    // |E|^2, contributions, V_t (into the context's real scratch), energy
    k_gpe_vbar<<<rg, kThreads, 0, st>>>(G + kGpeE * M, psi_grid, G + kGpeTot * M, phi_eps,
                                        contrib, T, M, eps_t, q_t, (float)(0.5 / e0inv), c->d_grid,
                                        elec_dot_out, c->gpe_ws, energy_out, c->d_box,
                                        0.5 / e0inv);
    HPF_LAUNCH_CHECK();
    if (psi_out)
        HPF_CUDA_TRY(cudaMemcpyAsync(psi_out, psi_grid, sizeof(float) * M,
                                     cudaMemcpyDeviceToDevice, st));
    if (elec_field_out)
        HPF_CUDA_TRY(cudaMemcpyAsync(elec_field_out, G + kGpeE * M, sizeof(float) * 3 * M,
                                     cudaMemcpyDeviceToDevice, st));
    if (vbar_out)
        HPF_CUDA_TRY(cudaMemcpyAsync(vbar_out, c->d_grid, sizeof(float) * T * M,
                                     cudaMemcpyDeviceToDevice, st));
    // forces: -grad (H * V_t) read out per type
    if ((r = exec_r2c(c, c->d_grid, c->d_spec_phi, T, st)) != HPF_OK) return r;
    k_gpe_force_spec<<<gk, kThreads, 0, st>>>(c->d_spec_phi, c->d_spec, T, Mc, g, c->d_box,
                                              c->d_fun);
    HPF_LAUNCH_CHECK();
    if ((r = exec_c2r(c, c->d_spec, c->d_grid, 3 * T, st)) != HPF_OK) return r;
    if (n > 0 &&
        (r = launch_readout(c, c->d_grid, pos, types, nullptr, n, T, elec_forces, nullptr, st)) !=
            HPF_OK)
        return r;
    if (iterations) {
        // the count of the loop just run (the one read-back of the call)
        HPF_CUDA_TRY(cudaMemcpyAsync(c->gpe_host, gpe_iter(c), sizeof(int),
                                     cudaMemcpyDeviceToHost, st));
        HPF_CUDA_TRY(cudaStreamSynchronize(st));
        memcpy(iterations, c->gpe_host, sizeof(int));
    }
    return HPF_OK;
}

// ------------------------------------------------- force vector-Jacobian ---
// Reverse-mode product of the field force with a cotangent lambda (N x 3):
// F_i = sum_g W(g - x_i) E_{t_i}(g), E_{t,d} = A_d H^2 (Q phi)_t with A_d the
// spectral derivative -i k'_d (antisymmetric), phi_j = m_j/dV sum W.  Then
//   d(lambda.F)/dx_j = sum_g grad W(g - x_j) (lambda_j . E_{t_j}(g))     (local)
//                    + m_{t_j}/dV sum_g U_{t_j}(g) grad W(g - x_j)      (global)
// with U_j = sum_{t,d} Q_jt H^2 (+i k'_d) rho_{t,d} and the lambda-weighted
// paint rho_{t,d}(g) = sum_{i in t} lambda_{i,d} W(g - x_i);
//   d(lambda.F)/dQ_tj = sum_d <rho_{t,d}, A_d H^2 phi_j>  (Parseval).
namespace {

__global__ void k_vjp_local(const float* __restrict__ E, const float* __restrict__ pos,
                            const int32_t* __restrict__ types, const float* __restrict__ lam,
                            int64_t n, int T, int64_t M, const BoxState* __restrict__ bs,
                            float* __restrict__ grad, int* err,
                            const float* __restrict__ charges = nullptr) {
    const int n0 = bs->n[0], n1 = bs->n[1], n2 = bs->n[2];
    const float h0 = bs->ih_hi[0], h1 = bs->ih_hi[1], h2 = bs->ih_hi[2];
    const float l0 = bs->ih_lo[0], l1 = bs->ih_lo[1], l2 = bs->ih_lo[2];
    const float i0 = h0 + l0, i1 = h1 + l1, i2 = h2 + l2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        const int t = types ? types[i] : 0;
        float gr[3] = {0.0f, 0.0f, 0.0f};
        const bool ok = isfinite(x) && isfinite(y) && isfinite(z) && t >= 0 && t < T;
        if (!ok) hpf_flag(err, (t >= 0 && t < T) ? HPF_ERR_NONFINITE : HPF_ERR_INDEX);
        if (ok) {
            int ix, iy, iz;
            float fx, fy, fz;
            grid_coord(x, h0, l0, n0, ix, fx);
            grid_coord(y, h1, l1, n1, iy, fy);
            grid_coord(z, h2, l2, n2, iz, fz);
            const int xs[2] = {ix, ix + 1 == n0 ? 0 : ix + 1};
            const int ys[2] = {iy, iy + 1 == n1 ? 0 : iy + 1};
            const int zs[2] = {iz, iz + 1 == n2 ? 0 : iz + 1};
            const float wx[2] = {1.0f - fx, fx}, wy[2] = {1.0f - fy, fy}, wz[2] = {1.0f - fz, fz};
            const float dx[2] = {-i0, i0}, dy[2] = {-i1, i1}, dz[2] = {-i2, i2};
            const float lx = lam[3 * i], ly = lam[3 * i + 1], lz = lam[3 * i + 2];
            const float* base = E + (int64_t)t * 3 * M;
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int b = 0; b < 2; ++b) {
                    const int64_t row = ((int64_t)xs[a] * n1 + ys[b]) * n2;
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        const int64_t o = row + zs[c];
                        const float v = fmaf(lx, __ldg(base + o),
                                             fmaf(ly, __ldg(base + M + o), lz * __ldg(base + 2 * M + o)));
                        gr[0] = fmaf(dx[a] * wy[b] * wz[c], v, gr[0]);
                        gr[1] = fmaf(wx[a] * dy[b] * wz[c], v, gr[1]);
                        gr[2] = fmaf(wx[a] * wy[b] * dz[c], v, gr[2]);
                    }
                }
        }
        // charges: F_i = q_i sum W E, so the local term carries q_i
        const float qq = charges ? charges[i] : 1.0f;
        grad[3 * i] = qq * gr[0];
        grad[3 * i + 1] = qq * gr[1];
        grad[3 * i + 2] = qq * gr[2];
    }
}

// rho[d][t][g] += lambda_{i,d} W(g - x_i) (float atomics)
__global__ void k_paint_lambda(const float* __restrict__ pos, const int32_t* __restrict__ types,
                               const float* __restrict__ lam, int64_t n, int T, int64_t M,
                               const BoxState* __restrict__ bs, float* __restrict__ rho,
                               const float* __restrict__ charges = nullptr) {
    const int n0 = bs->n[0], n1 = bs->n[1], n2 = bs->n[2];
    const float h0 = bs->ih_hi[0], h1 = bs->ih_hi[1], h2 = bs->ih_hi[2];
    const float l0 = bs->ih_lo[0], l1 = bs->ih_lo[1], l2 = bs->ih_lo[2];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        const int t = types ? types[i] : 0;
        if (!(isfinite(x) && isfinite(y) && isfinite(z)) || t < 0 || t >= T) continue;
        int ix, iy, iz;
        float fx, fy, fz;
        grid_coord(x, h0, l0, n0, ix, fx);
        grid_coord(y, h1, l1, n1, iy, fy);
        grid_coord(z, h2, l2, n2, iz, fz);
        const int xs[2] = {ix, ix + 1 == n0 ? 0 : ix + 1};
        const int ys[2] = {iy, iy + 1 == n1 ? 0 : iy + 1};
        const int zs[2] = {iz, iz + 1 == n2 ? 0 : iz + 1};
        const float wx[2] = {1.0f - fx, fx}, wy[2] = {1.0f - fy, fy}, wz[2] = {1.0f - fz, fz};
        // charges: the cotangent weighted by the bead's charge
        const float qq = charges ? charges[i] : 1.0f;
        if (qq == 0.0f) continue;
        const float l[3] = {qq * lam[3 * i], qq * lam[3 * i + 1], qq * lam[3 * i + 2]};
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                const int64_t row = ((int64_t)xs[a] * n1 + ys[b]) * n2;
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const float w = wx[a] * wy[b] * wz[c];
#pragma unroll
                    for (int d = 0; d < 3; ++d)
                        atomicAdd(rho + ((int64_t)d * T + t) * M + row + zs[c], w * l[d]);
                }
            }
    }
}

// U_j(k) = H^2/M sum_t Q_jt S_t, S_t = sum_d i k'_d rho_{d,t}(k), written over
// phi_k (read first); dQ_tj += w_k H^2/M Re(conj(S_t) phi_j(k))
template <int TT>
__global__ void k_vjp_kspace(const float2* __restrict__ rho_k, float2* phi_k, int64_t Mc,
                             KGeom g, const BoxState* __restrict__ bs,
                             const Functional* __restrict__ fun, double* dQ, double* partials,
                             unsigned int* ticket) {
    constexpr int K = TT * TT;
    float acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0f;
    const float s2h = fun->sigma2_half;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        float kx, ky, kz, gx, gy, gz, wk;
        mode_k(idx, g, bs, kx, ky, kz, gx, gy, gz, wk);
        const float H = expf(-s2h * (kx * kx + ky * ky + kz * kz));
        const float h2m = H * H * g.invM;
        const float gk[3] = {gx, gy, gz};
        float2 S[TT], ph[TT];
#pragma unroll
        for (int t = 0; t < TT; ++t) {
            float sx = 0.0f, sy = 0.0f;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const float2 r = rho_k[((int64_t)d * TT + t) * Mc + idx];
                sx = fmaf(-gk[d], r.y, sx);
                sy = fmaf(gk[d], r.x, sy);
            }
            S[t] = make_float2(sx, sy);
            ph[t] = phi_k[(int64_t)t * Mc + idx];
        }
        if (dQ) {
#pragma unroll
            for (int t = 0; t < TT; ++t)
#pragma unroll
                for (int j = 0; j < TT; ++j)
                    acc[t * TT + j] =
                        fmaf(wk * h2m, fmaf(S[t].x, ph[j].x, S[t].y * ph[j].y), acc[t * TT + j]);
        }
#pragma unroll
        for (int j = 0; j < TT; ++j) {
            float ux = 0.0f, uy = 0.0f;
#pragma unroll
            for (int t = 0; t < TT; ++t) {
                const float q = fun->Q[j * TT + t];
                ux = fmaf(q, S[t].x, ux);
                uy = fmaf(q, S[t].y, uy);
            }
            phi_k[(int64_t)j * Mc + idx] = make_float2(ux * h2m, uy * h2m);
        }
    }
    if (dQ) grid_reduce_store_f<K, kThreads>(acc, partials, ticket, dQ);
}

// Adjoint of the PIC map (hymd/field.py:356-403): E_d(k) = -i k'_d psi(k),
// psi = c M rho(k) / M with c(k) = 4 pi f H(k) / (M k^2) (k = 0: k^2 = 1, where
// k'_d = 0), so U(k) = c(k) sum_d i k'_d P_d(k) for the charge-weighted
// cotangent paint P_d (written over u_k).
__global__ void k_vjp_kspace_pic(const float2* __restrict__ p_k, float2* __restrict__ u_k,
                                 int64_t Mc, KGeom g, const BoxState* __restrict__ bs,
                                 const Functional* __restrict__ fun, float four_pi_fac) {
    const float s2h = fun->sigma2_half;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < Mc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        float kx, ky, kz, gx, gy, gz, wk;
        mode_k(idx, g, bs, kx, ky, kz, gx, gy, gz, wk);
        float k2 = kx * kx + ky * ky + kz * kz;
        const float H = expf(-s2h * k2);
        if (idx == 0) k2 = 1.0f;
        const float cc = four_pi_fac * H / k2 * g.invM;
        const float gk[3] = {gx, gy, gz};
        float sx = 0.0f, sy = 0.0f;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float2 r = p_k[(int64_t)d * Mc + idx];
            sx = fmaf(-gk[d], r.y, sx);
            sy = fmaf(gk[d], r.x, sy);
        }
        u_k[idx] = make_float2(cc * sx, cc * sy);
    }
}

}  // namespace

extern "C" int hpf_pic_force_vjp(hpf_ctx* c, const float* pos, const float* charges, int64_t n,
                                 double elec_factor, const float* lam, float* grad_pos,
                                 void* stream) {
    if (!c || n < 0 || (n > 0 && (!pos || !charges || !lam || !grad_pos))) return HPF_ERR_ARG;
    if (n == 0) return HPF_OK;
    cudaStream_t st = as_stream(stream);
    const int64_t M = c->M, Mc = c->Mc;
    const float four_pi_fac = (float)(4.0 * 3.14159265358979323846 * elec_factor);
    TypeScale sq;
    sq.s[0] = 1.0f;
    int r;
    // forward charge density, psi and E spectra, E grids
    if ((r = do_paint(c, pos, nullptr, charges, n, 1, sq, c->d_grid, st)) != HPF_OK) return r;
    if ((r = exec_r2c(c, c->d_grid, c->d_spec_phi, 1, st)) != HPF_OK) return r;
    const KGeom g = kgeom(c);
    k_kspace_pic<<<grid_for(Mc, kThreads), kThreads, 0, st>>>(
        c->d_spec_phi, c->d_spec, Mc, g, c->d_box, c->d_fun, four_pi_fac, nullptr, nullptr,
        nullptr);
    HPF_LAUNCH_CHECK();
    if ((r = exec_c2r(c, c->d_spec + Mc, c->d_grid, 3, st)) != HPF_OK) return r;
    k_vjp_local<<<grid_for(n, kThreads), kThreads, 0, st>>>(c->d_grid, pos, nullptr, lam, n, 1,
                                                            M, c->d_box, grad_pos, c->d_err,
                                                            charges);
    HPF_LAUNCH_CHECK();
    // charge-weighted cotangent paint [d][M], its spectra, U, and the readout
    HPF_CUDA_TRY(cudaMemsetAsync(c->d_grid, 0, sizeof(float) * 3 * M, st));
    k_paint_lambda<<<grid_for(n, kThreads), kThreads, 0, st>>>(pos, nullptr, lam, n, 1, M,
                                                               c->d_box, c->d_grid, charges);
    HPF_LAUNCH_CHECK();
    for (int d = 0; d < 3; ++d)
        if ((r = exec_r2c(c, c->d_grid + (int64_t)d * M, c->d_spec + (int64_t)d * Mc, 1, st)) !=
            HPF_OK)
            return r;
    k_vjp_kspace_pic<<<grid_for(Mc, kThreads), kThreads, 0, st>>>(
        c->d_spec, c->d_spec_phi, Mc, g, c->d_box, c->d_fun, four_pi_fac);
    HPF_LAUNCH_CHECK();
    if ((r = exec_c2r(c, c->d_spec_phi, c->d_grid, 1, st)) != HPF_OK) return r;
    k_readout_grad<<<grid_for(n, kThreads), kThreads, 0, st>>>(c->d_grid, pos, nullptr, n, 1, M,
                                                               c->d_box, sq, grad_pos, c->d_err,
                                                               1, 1, charges);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

extern "C" int hpf_field_force_vjp(hpf_ctx* c, const float* pos, const int32_t* types, int64_t n,
                                   const double* type_mass, const float* lam, float* grad_pos,
                                   double* dQ, void* stream) {
    if (!c || !type_mass || n < 0 || (n > 0 && (!pos || !types || !lam || !grad_pos)))
        return HPF_ERR_ARG;
    const int T = c->T;
    if (T > 8) return HPF_ERR_NOT_IMPLEMENTED;
    if (n == 0) return HPF_OK;
    cudaStream_t st = as_stream(stream);
    const int64_t M = c->M, Mc = c->Mc;
    TypeScale sc;
    for (int t = 0; t < T; ++t) sc.s[t] = (float)type_mass[t];
    int r;
    // forward force mesh E (kept raw spectra phi_k in d_spec_phi)
    if ((r = do_paint(c, pos, types, nullptr, n, T, sc, c->d_grid, st)) != HPF_OK) return r;
    if ((r = exec_r2c(c, c->d_grid, c->d_spec_phi, T, st)) != HPF_OK) return r;
    if ((r = launch_kspace_force(c, c->d_spec_phi, c->d_spec, nullptr, nullptr, nullptr, st)) !=
        HPF_OK)
        return r;
    if ((r = exec_c2r(c, c->d_spec, c->d_grid, 3 * T, st)) != HPF_OK) return r;
    k_vjp_local<<<grid_for(n, kThreads), kThreads, 0, st>>>(c->d_grid, pos, types, lam, n, T, M,
                                                            c->d_box, grad_pos, c->d_err);
    HPF_LAUNCH_CHECK();
    // lambda-weighted paint [d][t][M], its spectra, U, and the readout
    HPF_CUDA_TRY(cudaMemsetAsync(c->d_grid, 0, sizeof(float) * 3 * T * M, st));
    k_paint_lambda<<<grid_for(n, kThreads), kThreads, 0, st>>>(pos, types, lam, n, T, M,
                                                               c->d_box, c->d_grid);
    HPF_LAUNCH_CHECK();
    for (int d = 0; d < 3; ++d)
        if ((r = exec_r2c(c, c->d_grid + (int64_t)d * T * M, c->d_spec + (int64_t)d * T * Mc, T,
                          st)) != HPF_OK)
            return r;
    const KGeom g = kgeom(c);
    const int K = T * T;
    int grid = dQ ? reduce_grid(Mc, kThreads) : grid_for(Mc, kThreads);
    if (dQ && grid > 8 * HPF_REDUCE_BLOCKS / K) grid = 8 * HPF_REDUCE_BLOCKS / K;
    double* part = ws_partials(c->d_ws);
    unsigned int* tick = ws_ticket(c->d_ws);
#define HPF_VK(TT)                                                                         \
    k_vjp_kspace<TT><<<grid, kThreads, 0, st>>>(c->d_spec, c->d_spec_phi, Mc, g, c->d_box, \
                                                c->d_fun, dQ, part, tick)
    switch (T) {
        case 1: HPF_VK(1); break;
        case 2: HPF_VK(2); break;
        case 3: HPF_VK(3); break;
        case 4: HPF_VK(4); break;
        case 5: HPF_VK(5); break;
        case 6: HPF_VK(6); break;
        case 7: HPF_VK(7); break;
        default: HPF_VK(8); break;
    }
#undef HPF_VK
    HPF_LAUNCH_CHECK();
    if ((r = exec_c2r(c, c->d_spec_phi, c->d_grid, T, st)) != HPF_OK) return r;
    k_readout_grad<<<grid_for(n, kThreads), kThreads, 0, st>>>(c->d_grid, pos, types, n, T, M,
                                                               c->d_box, sc, grad_pos, c->d_err,
                                                               1, 1);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

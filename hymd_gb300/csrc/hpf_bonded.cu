// Bonded forces of HyMD on GB300: harmonic bonds, harmonic angles, cosine-
// series / combined bending-torsion / improper dihedrals with the peptide
// dipole reconstruction, and the redistribution of dipole forces.
//
// Reference behaviour (paths inside the HyMD project):
//   cbf   hymd/compute_bond_forces.f90:1-61
//   caf   hymd/compute_angle_forces.f90:1-93
//   cdf   hymd/compute_dihedral_forces.f90:1-137
//   cosine_series, reconstruct   hymd/dipole_reconstruction.f90:37-220
//   dipole_forces_redistribution hymd/force.py:855-877
//
// One thread per term.  Differences of stored positions are taken in FP32,
// exactly as the Fortran does (real(4) operands); the per-term arithmetic is
// FP32 (GB300's FP64 rate is far too low for a hot path) with formulations
// that stay well conditioned where the Fortran's FP64 acos would not:
// angles use atan2(|e_a x e_c|, e_a . e_c).  Energies and virials are summed
// in FP64 by a deterministic grid reduction; forces are accumulated with FP32
// atomics.
#include <math.h>

#include "hpf_internal.cuh"

namespace {

constexpr int kThreads = 256;

struct V3 {
    float x, y, z;
};

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float norm(V3 a) { return sqrtf(dot(a, a)); }

struct Box {
    float L[3], iL[3];
};

__device__ __forceinline__ Box load_box(const double* box) {
    Box b;
    for (int d = 0; d < 3; ++d) {
        b.L[d] = (float)box[d];
        b.iL[d] = (float)(1.0 / box[d]);
    }
    return b;
}

// rab - box * nint(rab / box); nint rounds half away from zero (roundf).
__device__ __forceinline__ V3 min_image(V3 r, const Box& b) {
    r.x = fmaf(-b.L[0], roundf(r.x * b.iL[0]), r.x);
    r.y = fmaf(-b.L[1], roundf(r.y * b.iL[1]), r.y);
    r.z = fmaf(-b.L[2], roundf(r.z * b.iL[2]), r.z);
    return r;
}

__device__ __forceinline__ V3 load3(const float* r, int i) {
    return v3(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
}

__device__ __forceinline__ void add3(float* f, int i, V3 v) {
    atomicAdd(f + 3 * i, v.x);
    atomicAdd(f + 3 * i + 1, v.y);
    atomicAdd(f + 3 * i + 2, v.z);
}

__device__ __forceinline__ bool in_range(int i, int64_t n) { return i >= 0 && (int64_t)i < n; }

// ------------------------------------------------------------------ bonds ---
__global__ void k_bonds(float* __restrict__ f, const float* __restrict__ r, int64_t n,
                        const double* __restrict__ box, const int32_t* __restrict__ a,
                        const int32_t* __restrict__ b, const float* __restrict__ r0,
                        const float* __restrict__ kk, int64_t nb, double* out, int* err) {
    const Box bx = load_box(box);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nb;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int ia = a[i], ib = b[i];
        if (!in_range(ia, n) || !in_range(ib, n)) {
            hpf_flag(err, HPF_ERR_INDEX);
            continue;
        }
        const V3 rab = min_image(load3(r, ib) - load3(r, ia), bx);
        const float rn = norm(rab);
        const float dr = rn - r0[i];
        const float df = kk[i] * dr;
        const V3 fa = (-df / rn) * rab;
        add3(f, ia, -fa);
        add3(f, ib, fa);
        acc[0] += 0.5 * (double)(kk[i] * dr) * (double)dr;
        acc[1] += (double)(fa.x * rab.x);
        acc[2] += (double)(fa.y * rab.y);
        acc[3] += (double)(fa.z * rab.z);
    }
    grid_reduce_store<4>(acc, ws_partials(out), ws_ticket(out), out, false);
}

// ----------------------------------------------------------------- angles ---
__global__ void k_angles(float* __restrict__ f, const float* __restrict__ r, int64_t n,
                         const double* __restrict__ box, const int32_t* __restrict__ a,
                         const int32_t* __restrict__ b, const int32_t* __restrict__ c,
                         const float* __restrict__ t0, const float* __restrict__ kk, int64_t na,
                         double* out, int* err) {
    const Box bx = load_box(box);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < na;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int ia = a[i], ib = b[i], ic = c[i];
        if (!in_range(ia, n) || !in_range(ib, n) || !in_range(ic, n)) {
            hpf_flag(err, HPF_ERR_INDEX);
            continue;
        }
        const V3 rb = load3(r, ib);
        const V3 ra = min_image(load3(r, ia) - rb, bx);
        const V3 rc = min_image(load3(r, ic) - rb, bx);
        const float na_ = norm(ra), nc_ = norm(rc);
        const V3 ea = (1.0f / na_) * ra, ec = (1.0f / nc_) * rc;
        const float cosphi = dot(ea, ec);
        const float sinphi = norm(cross(ea, ec));
        if (!(sinphi > 0.0f)) continue;  // collinear: the Fortran skips cos^2 >= 1
        const float theta = atan2f(sinphi, cosphi);
        const float d = theta - t0[i];
        const float ff = kk[i] * d;
        const float xa = -ff / (na_ * sinphi), xc = -ff / (nc_ * sinphi);
        const V3 fa = xa * (ec - cosphi * ea);
        const V3 fc = xc * (ea - cosphi * ec);
        add3(f, ia, -fa);
        add3(f, ic, -fc);
        add3(f, ib, fa + fc);
        acc[0] += 0.5 * (double)ff * (double)d;
        acc[1] -= (double)(fa.x * ra.x) + (double)(fc.x * rc.x);
        acc[2] -= (double)(fa.y * ra.y) + (double)(fc.y * rc.y);
        acc[3] -= (double)(fa.z * ra.z) + (double)(fc.z * rc.z);
    }
    grid_reduce_store<4>(acc, ws_partials(out), ws_ticket(out), out, false);
}

// -------------------------------------------------------------- dihedrals ---
__device__ __forceinline__ void cosine_series(const float* cn, const float* dn, float phi,
                                              float& e, float& de) {
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        float s, c;
        sincosf(i * phi - dn[i], &s, &c);
        e = fmaf(cn[i], 1.0f + c, e);
        de = fmaf(-(float)i * cn[i], s, de);
    }
}

// reconstruct (dipole_reconstruction.f90:50-220): CBT bending energy of the
// angle (rab, rcb) at bead rb and, with dipole_flag, the two dipole
// pseudo-charge positions and the three 3x3 transfer matrices.  Outputs are
// the positive gradients fa, fb, fc.  Where cos^2(gamma) >= 1 the Fortran
// leaves its outputs unassigned; here they are zero.
__device__ void reconstruct(V3 rab, V3 rb, V3 rcb, const Box& bx, const float* c_k,
                            const float* d_k, float phi, int dipole_flag, float& e_cbt,
                            float& df_cbt, V3& fa, V3& fb, V3& fc, float* dipole, float* tm) {
    // cos(1.392947) / sin(1.392947): single-precision literals in the Fortran
    const float cos_psi = cosf(1.392947f), sin_psi = sinf(1.392947f);
    const float delta = 0.3f;
    float k = 0.0f, dk = 0.0f;
    const float gamma_0 = 1.85f - 0.227f * cosf(phi - 0.785f);
    const float dg = 0.227f * sinf(phi - 0.785f);
    cosine_series(c_k, d_k, phi, k, dk);
    const float norm_a = norm(rab), norm_c = norm(rcb);
    const V3 w = (1.0f / norm_a) * rab, v = (1.0f / norm_c) * rcb;
    const float cos_gamma = dot(w, v);
    e_cbt = 0.0f;
    df_cbt = 0.0f;
    fa = fb = fc = v3(0.f, 0.f, 0.f);
    if (!(cos_gamma * cos_gamma < 1.0f)) return;
    const float gamm = acosf(cos_gamma);
    float sin_gamma = sqrtf(1.0f - cos_gamma * cos_gamma);
    if (sin_gamma < 0.1f) sin_gamma = 0.1f;
    fa = (-1.0f / (norm_a * sin_gamma)) * (v - cos_gamma * w);
    fc = (-1.0f / (norm_c * sin_gamma)) * (w - cos_gamma * v);
    fb = -(fa + fc);
    const float df_ang = k * (gamm - gamma_0);
    const float var_sq = (gamm - gamma_0) * (gamm - gamma_0);
    e_cbt = 0.5f * k * var_sq;
    df_cbt = 0.5f * dk * var_sq - df_ang * dg;
    if (dipole_flag) {
        const float fac = expf((gamm - 1.73f) / 0.025f);
        const float theta = -1.607f * gamm + 0.094f + 1.883f / (1.0f + fac);
        const float d_theta = -1.607f - 1.883f / 0.025f * fac / ((1.0f + fac) * (1.0f + fac));
        float sin_theta, cos_theta;
        sincosf(theta, &sin_theta, &cos_theta);
        const V3 nn = (1.0f / sin_gamma) * cross(w, v);
        const V3 m = cross(nn, v);
        const V3 r0 = rb + 0.5f * rcb;
        const V3 d = (0.5f * delta) * (cos_psi * v + sin_psi * (cos_theta * nn + sin_theta * m));
        const V3 p[2] = {r0 + d, r0 - d};
        for (int q = 0; q < 2; ++q) {
            const V3 pw = min_image(p[q], bx);
            dipole[3 * q] = pw.x;
            dipole[3 * q + 1] = pw.y;
            dipole[3 * q + 2] = pw.z;
        }
        const float wv[3] = {w.x, w.y, w.z}, vv[3] = {v.x, v.y, v.z};
        const float nv[3] = {nn.x, nn.y, nn.z}, mv[3] = {m.x, m.y, m.z};
        const float fav[3] = {fa.x, fa.y, fa.z}, fbv[3] = {fb.x, fb.y, fb.z},
                    fcv[3] = {fc.x, fc.y, fc.z};
        float Vb[3][3], Wb[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                Vb[i][j] = (vv[i] * vv[j] - (i == j ? 1.0f : 0.0f)) / norm_c;
                Wb[i][j] = (wv[i] * wv[j] - (i == j ? 1.0f : 0.0f)) / norm_a;
            }
        // cross_matrix(Mx, x): row i = cross(Mx(i,:), x); with Vc = -Vb, Wa = -Wb
        for (int i = 0; i < 3; ++i) {
            const V3 Wbi = v3(Wb[i][0], Wb[i][1], Wb[i][2]);
            const V3 Vbi = v3(Vb[i][0], Vb[i][1], Vb[i][2]);
            const V3 cWb_v = cross(Wbi, v), cVb_w = cross(Vbi, w), cVb_n = cross(Vbi, nn);
            // N rows (S19): N_a = (cos g fa n^T - cross(Wb, v)) / sin g, etc.
            const V3 nvec = nn;
            const V3 Na = (1.0f / sin_gamma) * (cos_gamma * fav[i] * nvec - cWb_v);
            const V3 Nb = (1.0f / sin_gamma) * (cos_gamma * fbv[i] * nvec + cWb_v - cVb_w);
            const V3 Nc = (1.0f / sin_gamma) * (cos_gamma * fcv[i] * nvec + cVb_w);
            const V3 Ma = cross(Na, v);
            const V3 Mb = cross(Nb, v) - cVb_n;
            const V3 Mc = cross(Nc, v) + cVb_n;
            const float Ma_[3] = {Ma.x, Ma.y, Ma.z}, Mb_[3] = {Mb.x, Mb.y, Mb.z},
                        Mc_[3] = {Mc.x, Mc.y, Mc.z};
            const float Na_[3] = {Na.x, Na.y, Na.z}, Nb_[3] = {Nb.x, Nb.y, Nb.z},
                        Nc_[3] = {Nc.x, Nc.y, Nc.z};
            for (int j = 0; j < 3; ++j) {
                const float st_dt = sin_theta * d_theta, ct_dt = cos_theta * d_theta;
                const float FNa = st_dt * fav[i] * nv[j], FMa = ct_dt * fav[i] * mv[j];
                const float FNb = st_dt * fbv[i] * nv[j], FMb = ct_dt * fbv[i] * mv[j];
                const float FNc = st_dt * fcv[i] * nv[j], FMc = ct_dt * fcv[i] * mv[j];
                tm[0 * 9 + i * 3 + j] =
                    0.5f * delta * (sin_psi * (cos_theta * Na_[j] + sin_theta * Ma_[j] + FNa - FMa));
                tm[1 * 9 + i * 3 + j] =
                    0.5f * delta * (cos_psi * Vb[i][j] +
                                    sin_psi * (cos_theta * Nb_[j] + sin_theta * Mb_[j] + FNb - FMb));
                tm[2 * 9 + i * 3 + j] =
                    0.5f * delta * (-cos_psi * Vb[i][j] +
                                    sin_psi * (cos_theta * Nc_[j] + sin_theta * Mc_[j] + FNc - FMc));
            }
        }
    }
    fa = df_ang * fa;
    fb = df_ang * fb;
    fc = df_ang * fc;
}

__global__ void k_dihedrals(float* __restrict__ force, const float* __restrict__ r, int64_t n,
                            float* __restrict__ dipoles, float* __restrict__ transfer,
                            const double* __restrict__ box, const int32_t* __restrict__ a,
                            const int32_t* __restrict__ b, const int32_t* __restrict__ c,
                            const int32_t* __restrict__ d, const float* __restrict__ coeff,
                            const int32_t* __restrict__ dtype, const int32_t* __restrict__ last,
                            int64_t nd, int dipole_flag, double* out, int* err) {
    const Box bx = load_box(box);
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
         i += (int64_t)gridDim.x * blockDim.x) {
        float* dip = dipoles ? dipoles + 12 * i : nullptr;
        float* tmx = transfer ? transfer + 54 * i : nullptr;
        if (dip)
            for (int q = 0; q < 12; ++q) dip[q] = 0.0f;
        if (tmx)
            for (int q = 0; q < 54; ++q) tmx[q] = 0.0f;
        const int ia = a[i], ib = b[i], ic = c[i], id = d[i];
        if (!in_range(ia, n) || !in_range(ib, n) || !in_range(ic, n) || !in_range(id, n)) {
            hpf_flag(err, HPF_ERR_INDEX);
            continue;
        }
        const V3 pa = load3(r, ia), pb = load3(r, ib), pc = load3(r, ic), pd = load3(r, id);
        const V3 fv = min_image(pa - pb, bx);
        const V3 g = min_image(pb - pc, bx);
        const V3 h = min_image(pd - pc, bx);
        const V3 v = cross(fv, g), w = cross(h, g);
        const float v_sq = dot(v, v), w_sq = dot(w, w);
        const float g_norm = norm(g);
        const float cos_phi = dot(v, w);
        const float sin_phi = dot(w, fv) * g_norm;
        const float phi = atan2f(sin_phi, cos_phi);
        const float f_dot_g = dot(fv, g), h_dot_g = dot(h, g);
        const int ty = dtype[i];
        float row[6][5];
        const float* cf = coeff + 30 * i;
        for (int p = 0; p < 6; ++p)
            for (int q = 0; q < 5; ++q) row[p][q] = cf[5 * p + q];
        float e = 0.0f, df_dih = 0.0f;
        if (ty == 0 || ty == 1) {
            cosine_series(row[0], row[1], phi, e, df_dih);
            bool nz_c = false, nz_d = false;
            for (int q = 0; q < 5; ++q) {
                nz_c |= row[2][q] != 0.0f;
                nz_d |= row[3][q] != 0.0f;
            }
            if (nz_c && nz_d) cosine_series(row[2], row[3], phi, e, df_dih);
        }
        if (ty == 1) {
            float e_cbt, df_cbt;
            V3 fa, fb, fc, fd;
            reconstruct(fv, pb, -g, bx, row[4], row[5], phi, dipole_flag, e_cbt, df_cbt, fa, fb,
                        fc, dip, tmx);
            e += e_cbt;
            df_dih += df_cbt;
            add3(force, ia, -fa);
            add3(force, ib, -fb);
            add3(force, ic, -fc);
            if (last[i] == 1) {
                reconstruct(g, pc, h, bx, row[4], row[5], phi, dipole_flag, e_cbt, df_cbt, fb, fc,
                            fd, dip ? dip + 6 : nullptr, tmx ? tmx + 27 : nullptr);
                e += e_cbt;
                df_dih += df_cbt;
                add3(force, ib, -fb);
                add3(force, ic, -fc);
                add3(force, id, -fd);
            }
        }
        if (ty == 2) {
            const float eq = row[0][0], kc = row[0][1];
            df_dih = kc * (phi - eq);
            e += 0.5f * kc * (phi - eq) * (phi - eq);
        }
        const V3 sc = (f_dot_g / (v_sq * g_norm)) * v - (h_dot_g / (w_sq * g_norm)) * w;
        const V3 fa = (-df_dih * g_norm / v_sq) * v;
        const V3 fd = (df_dih * g_norm / w_sq) * w;
        const V3 fb = df_dih * sc - fa;
        const V3 fc = -df_dih * sc - fd;
        add3(force, ia, fa);
        add3(force, ib, fb);
        add3(force, ic, fc);
        add3(force, id, fd);
        acc[0] += (double)e;
    }
    grid_reduce_store<1>(acc, ws_partials(out), ws_ticket(out), out, false);
}

// --------------------------------------------------- dipole redistribution ---
__global__ void k_dipole_redistribute(float* __restrict__ fob, int64_t n,
                                      const float* __restrict__ fdip,
                                      const float* __restrict__ tm, const int32_t* __restrict__ a,
                                      const int32_t* __restrict__ b, const int32_t* __restrict__ c,
                                      const int32_t* __restrict__ d,
                                      const int32_t* __restrict__ dtype,
                                      const int32_t* __restrict__ last, int64_t nd) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (dtype[i] != 1) continue;
        const int idx[4] = {a[i], b[i], c[i], d[i]};
        bool ok = true;
        for (int q = 0; q < 4; ++q) ok &= in_range(idx[q], n);
        if (!ok) continue;
        const float* fd = fdip + 12 * i;
        const float* m = tm + 54 * i;
        const int npair = last[i] == 1 ? 2 : 1;
        for (int pr = 0; pr < npair; ++pr) {
            const V3 f0 = v3(fd[6 * pr], fd[6 * pr + 1], fd[6 * pr + 2]);
            const V3 f1 = v3(fd[6 * pr + 3], fd[6 * pr + 4], fd[6 * pr + 5]);
            const V3 s = f0 + f1, df = f0 - f1;
            // atoms (a, b, c) for the first pair, (b, c, d) for the last angle
            for (int q = 0; q < 3; ++q) {
                const float* M = m + 27 * pr + 9 * q;
                V3 o = v3(M[0] * df.x + M[1] * df.y + M[2] * df.z,
                          M[3] * df.x + M[4] * df.y + M[5] * df.z,
                          M[6] * df.x + M[7] * df.y + M[8] * df.z);
                if (q > 0) o = o + 0.5f * s;
                add3(fob, idx[pr + q], o);
            }
        }
    }
}

int grid_for(int64_t work) {
    int64_t g = (work + kThreads - 1) / kThreads;
    if (g < 1) g = 1;
    if (g > HPF_REDUCE_BLOCKS) g = HPF_REDUCE_BLOCKS;
    return (int)g;
}

}  // namespace

extern "C" {

int hpf_bonds(float* f, const float* r, int64_t n, const double* box, const int32_t* a,
              const int32_t* b, const float* r0, const float* k, int64_t nb, double* out,
              int* d_err, void* stream) {
    if (!f || !r || !box || !out || n < 0 || nb < 0 || (nb > 0 && (!a || !b || !r0 || !k)))
        return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    HPF_CUDA_TRY(cudaMemsetAsync(f, 0, sizeof(float) * 3 * n, st));
    k_bonds<<<grid_for(nb), kThreads, 0, st>>>(f, r, n, box, a, b, r0, k, nb, out, d_err);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_angles(float* f, const float* r, int64_t n, const double* box, const int32_t* a,
               const int32_t* b, const int32_t* c, const float* t0, const float* k, int64_t na,
               double* out, int* d_err, void* stream) {
    if (!f || !r || !box || !out || n < 0 || na < 0 ||
        (na > 0 && (!a || !b || !c || !t0 || !k)))
        return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    HPF_CUDA_TRY(cudaMemsetAsync(f, 0, sizeof(float) * 3 * n, st));
    k_angles<<<grid_for(na), kThreads, 0, st>>>(f, r, n, box, a, b, c, t0, k, na, out, d_err);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_dihedrals(float* f, const float* r, int64_t n, float* dipoles, float* transfer,
                  const double* box, const int32_t* a, const int32_t* b, const int32_t* c,
                  const int32_t* d, const float* coeff, const int32_t* dtype,
                  const int32_t* last, int64_t nd, int dipole_flag, double* out, int* d_err,
                  void* stream) {
    if (!f || !r || !box || !out || n < 0 || nd < 0 ||
        (nd > 0 && (!a || !b || !c || !d || !coeff || !dtype || !last)))
        return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    HPF_CUDA_TRY(cudaMemsetAsync(f, 0, sizeof(float) * 3 * n, st));
    k_dihedrals<<<grid_for(nd), kThreads, 0, st>>>(f, r, n, dipoles, transfer, box, a, b, c, d,
                                                   coeff, dtype, last, nd, dipole_flag, out,
                                                   d_err);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_dipole_redistribute(float* f_on_bead, int64_t n, const float* f_dipoles,
                            const float* transfer, const int32_t* a, const int32_t* b,
                            const int32_t* c, const int32_t* d, const int32_t* dtype,
                            const int32_t* last, int64_t nd, void* stream) {
    if (!f_on_bead || n < 0 || nd < 0 ||
        (nd > 0 && (!f_dipoles || !transfer || !a || !b || !c || !d || !dtype || !last)))
        return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    HPF_CUDA_TRY(cudaMemsetAsync(f_on_bead, 0, sizeof(float) * 3 * n, st));
    if (nd > 0) {
        k_dipole_redistribute<<<grid_for(nd), kThreads, 0, st>>>(f_on_bead, n, f_dipoles,
                                                                 transfer, a, b, c, d, dtype,
                                                                 last, nd);
        HPF_LAUNCH_CHECK();
    }
    return HPF_OK;
}

}  // extern "C"

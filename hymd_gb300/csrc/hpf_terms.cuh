// Per-term bonded arithmetic shared by the stand-alone bonded kernels and the
// fused rRESPA kernel.  Each function takes the term's bead positions and
// returns the forces on its beads (no memory traffic of its own).
//
// Reference behaviour (paths inside the HyMD project):
//   cbf   hymd/compute_bond_forces.f90:45-61
//   caf   hymd/compute_angle_forces.f90:58-92
//   cdf   hymd/compute_dihedral_forces.f90:29-135
//   cosine_series / reconstruct  hymd/dipole_reconstruction.f90:37-220
// Differences of stored positions are taken in FP32 as the Fortran does
// (real(4) operands); the rest is FP32 arithmetic formulated to stay well
// conditioned: angles use atan2(|e_a x e_c|, e_a . e_c) instead of acos.
#pragma once

#include <math.h>

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

// The reciprocal only picks the periodic image (nint(r / L)), so FP32 is
// enough; an FP64 division per thread would keep GB300's thin FP64 pipe busy.
__device__ __forceinline__ Box load_box(const double* box) {
    Box b;
    for (int d = 0; d < 3; ++d) {
        b.L[d] = (float)box[d];
        b.iL[d] = 1.0f / b.L[d];
    }
    return b;
}

// r - box * nint(r / box); nint rounds half away from zero (roundf).
__device__ __forceinline__ V3 min_image(V3 r, const Box& b) {
    r.x = fmaf(-b.L[0], roundf(r.x * b.iL[0]), r.x);
    r.y = fmaf(-b.L[1], roundf(r.y * b.iL[1]), r.y);
    r.z = fmaf(-b.L[2], roundf(r.z * b.iL[2]), r.z);
    return r;
}

// Harmonic bond between a and b.  Returns the force on b (minus on a);
// e = 1/2 k (|r|-r0)^2; vir = fa * rab (componentwise, bond_pr).  Lengths
// and their reciprocals come from one rsqrt (<= 2 ulp), which keeps the term
// free of divisions.
__device__ __forceinline__ V3 bond_term(V3 pa, V3 pb, float r0, float k, const Box& bx,
                                        float& e, V3& vir) {
    const V3 rab = min_image(pb - pa, bx);
    const float d2 = dot(rab, rab);
    const float ir = rsqrtf(d2);
    const float rn = d2 * ir;
    const float dr = rn - r0;
    const V3 fa = (-k * dr * ir) * rab;
    e = 0.5f * k * dr * dr;
    vir = v3(fa.x * rab.x, fa.y * rab.y, fa.z * rab.z);
    return fa;
}

// Harmonic angle a-b-c.  Writes the positive gradients ga (on a) and gc (on
// c); the force on a is -ga, on c -gc, on b ga+gc.  Returns false for an
// exactly collinear triple (skipped, as the Fortran skips cos^2 >= 1).
__device__ __forceinline__ bool angle_term(V3 pa, V3 pb, V3 pc, float t0, float k, const Box& bx,
                                           V3& ga, V3& gc, float& e, V3& vir) {
    const V3 ra = min_image(pa - pb, bx);
    const V3 rc = min_image(pc - pb, bx);
    const float ia = rsqrtf(dot(ra, ra)), ic = rsqrtf(dot(rc, rc));
    const V3 ea = ia * ra, ec = ic * rc;
    const float cosphi = dot(ea, ec);
    const V3 cr = cross(ea, ec);
    const float s2 = dot(cr, cr);
    if (!(s2 > 0.0f)) return false;
    const float is = rsqrtf(s2);
    const float sinphi = s2 * is;
    const float theta = atan2f(sinphi, cosphi);
    const float d = theta - t0;
    const float ff = k * d;
    ga = (-ff * ia * is) * (ec - cosphi * ea);
    gc = (-ff * ic * is) * (ea - cosphi * ec);
    e = 0.5f * ff * d;
    vir = v3(-(ga.x * ra.x) - (gc.x * rc.x), -(ga.y * ra.y) - (gc.y * rc.y),
             -(ga.z * ra.z) - (gc.z * rc.z));
    return true;
}

// f / m for a fixed m with a precomputed reciprocal: one product and one FMA
// correction step (Markstein), which gives the correctly rounded quotient
// except in rare ties -- the FP32 F/m of the reference's integrate_velocity.
__device__ __forceinline__ float div_m(float f, float m, float inv_m) {
    const float q = f * inv_m;
    const float r = fmaf(-q, m, f);
    return fmaf(r, inv_m, q);
}

// cos and sin of the phase angles of a four-body term's coefficient rows 1,
// 3 and 5 (the d_n of the cosine series): trig[5r + q] = cos(row[2r+1][q]),
// trig[15 + 5r + q] = sin(row[2r+1][q]), r = 0, 1, 2.  They depend on the
// coefficients only, so the fused kernel's plan holds them once.
__device__ __forceinline__ void dih_phase_trig(const float* cf, float* trig) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            float sn, cs;
            sincosf(cf[5 * (2 * r + 1) + q], &sn, &cs);
            trig[5 * r + q] = cs;
            trig[15 + 5 * r + q] = sn;
        }
    }
}

// cos(n phi), sin(n phi) for n = 0..4 from cos phi and sin phi by the
// rotation recurrence (no trigonometric calls).
__device__ __forceinline__ void multiples(float cphi, float sphi, float (&C)[5], float (&S)[5]) {
    C[0] = 1.0f;
    S[0] = 0.0f;
#pragma unroll
    for (int n = 1; n < 5; ++n) {
        C[n] = fmaf(C[n - 1], cphi, -S[n - 1] * sphi);
        S[n] = fmaf(S[n - 1], cphi, C[n - 1] * sphi);
    }
}

// sum_n c_n (1 + cos(n phi - d_n)) into e and its phi-derivative
// sum_n -n c_n sin(n phi - d_n) into de, with cos(n phi - d) = C cos d +
// S sin d and sin(n phi - d) = S cos d - C sin d (cd, sd: the phases' cos,
// sin).
__device__ __forceinline__ void cosine_series(const float* cn, const float* cd, const float* sd,
                                              const float (&C)[5], const float (&S)[5],
                                              float& e, float& de) {
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const float c = fmaf(C[i], cd[i], S[i] * sd[i]);
        const float sn = fmaf(S[i], cd[i], -C[i] * sd[i]);
        e = fmaf(cn[i], 1.0f + c, e);
        de = fmaf(-(float)i * cn[i], sn, de);
    }
}

// The dipole pseudo-charge positions (dipole[0..5]) and the three 3x3
// transfer matrices (tm[0..26]) of reconstruct (dipole_reconstruction.f90:
// 107-220), from the unit bond vectors w, v, the angle gamma and the
// (not yet stiffness-scaled) angle gradients fa, fb, fc.  Only the last
// inner step asks for them, so this stays out of line.
static __device__ __noinline__ void dipole_transfer(V3 w, V3 v, V3 rb, V3 rcb, float norm_a,
                                                    float norm_c, float cos_gamma,
                                                    float sin_gamma, float gamm, V3 fa, V3 fb,
                                                    V3 fc, const Box& bx, float* dipole,
                                                    float* tm) {
    const float delta = 0.3f;
    // cos(1.392947) / sin(1.392947): single-precision literals in the Fortran
    const float cos_psi = cosf(1.392947f), sin_psi = sinf(1.392947f);
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
    for (int i = 0; i < 3; ++i) {
        float Vb[3], Wb[3];
        for (int j = 0; j < 3; ++j) {
            Vb[j] = (vv[i] * vv[j] - (i == j ? 1.0f : 0.0f)) / norm_c;
            Wb[j] = (wv[i] * wv[j] - (i == j ? 1.0f : 0.0f)) / norm_a;
        }
        // cross_matrix(Mx, x): row i = cross(Mx(i,:), x); with Vc = -Vb, Wa = -Wb
        const V3 Wbi = v3(Wb[0], Wb[1], Wb[2]);
        const V3 Vbi = v3(Vb[0], Vb[1], Vb[2]);
        const V3 cWb_v = cross(Wbi, v), cVb_w = cross(Vbi, w), cVb_n = cross(Vbi, nn);
        const V3 Na = (1.0f / sin_gamma) * (cos_gamma * fav[i] * nn - cWb_v);
        const V3 Nb = (1.0f / sin_gamma) * (cos_gamma * fbv[i] * nn + cWb_v - cVb_w);
        const V3 Nc = (1.0f / sin_gamma) * (cos_gamma * fcv[i] * nn + cVb_w);
        const V3 Ma = cross(Na, v);
        const V3 Mb = cross(Nb, v) - cVb_n;
        const V3 Mc = cross(Nc, v) + cVb_n;
        const float Ma_[3] = {Ma.x, Ma.y, Ma.z}, Mb_[3] = {Mb.x, Mb.y, Mb.z},
                    Mc_[3] = {Mc.x, Mc.y, Mc.z};
        const float Na_[3] = {Na.x, Na.y, Na.z}, Nb_[3] = {Nb.x, Nb.y, Nb.z},
                    Nc_[3] = {Nc.x, Nc.y, Nc.z};
        const float st_dt = sin_theta * d_theta, ct_dt = cos_theta * d_theta;
        for (int j = 0; j < 3; ++j) {
            const float FNa = st_dt * fav[i] * nv[j], FMa = ct_dt * fav[i] * mv[j];
            const float FNb = st_dt * fbv[i] * nv[j], FMb = ct_dt * fbv[i] * mv[j];
            const float FNc = st_dt * fcv[i] * nv[j], FMc = ct_dt * fcv[i] * mv[j];
            tm[0 * 9 + i * 3 + j] =
                0.5f * delta * (sin_psi * (cos_theta * Na_[j] + sin_theta * Ma_[j] + FNa - FMa));
            tm[1 * 9 + i * 3 + j] =
                0.5f * delta * (cos_psi * Vb[j] +
                                sin_psi * (cos_theta * Nb_[j] + sin_theta * Mb_[j] + FNb - FMb));
            tm[2 * 9 + i * 3 + j] =
                0.5f * delta * (-cos_psi * Vb[j] +
                                sin_psi * (cos_theta * Nc_[j] + sin_theta * Mc_[j] + FNc - FMc));
        }
    }
}

// reconstruct (dipole_reconstruction.f90:50-220): CBT bending energy of the
// angle (rab, rcb) at bead rb and, with dipole_flag, the two dipole
// pseudo-charge positions (dipole[0..5]) and the three 3x3 transfer matrices
// (tm[0..26]).  Outputs the positive gradients fa, fb, fc.  Where
// cos^2(gamma) >= 1 the Fortran leaves its outputs unassigned; here they are
// zero.
// The bending stiffness K(phi) is the cosine series of rows 4 (c_k) and 5
// (phases, as cos cd_k / sin sd_k); gamma_0(phi) = 1.85 - 0.227 cos(phi -
// 0.785) and its derivative come from cos phi, sin phi and the constants
// cos(0.785f), sin(0.785f).
static __device__ void reconstruct(V3 rab, V3 rb, V3 rcb, const Box& bx, const float* c_k,
                                   const float* cd_k, const float* sd_k, float cphi, float sphi,
                                   const float (&C)[5], const float (&S)[5], int dipole_flag,
                                   float& e_cbt, float& df_cbt, V3& fa, V3& fb, V3& fc,
                                   float* dipole, float* tm) {
    constexpr float c785 = 7.073882506e-01f, s785 = 7.068251997e-01f;  // cos, sin of 0.785f
    float k = 0.0f, dk = 0.0f;
    const float gamma_0 = 1.85f - 0.227f * fmaf(cphi, c785, sphi * s785);
    const float dg = 0.227f * fmaf(sphi, c785, -cphi * s785);
    cosine_series(c_k, cd_k, sd_k, C, S, k, dk);
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
    if (dipole_flag && dipole)
        dipole_transfer(w, v, rb, rcb, norm_a, norm_c, cos_gamma, sin_gamma, gamm, fa, fb, fc, bx,
                        dipole, tm);
    fa = df_ang * fa;
    fb = df_ang * fb;
    fc = df_ang * fc;
}

// Four-body term a-b-c-d of type ty (0 cosine series, 1 + CBT, 2 improper).
// coeff: 30 floats (6 rows x 5); trig: the 30 cos / sin of its phase rows
// (dih_phase_trig).  Writes the forces on the four beads (F[0..3]) and the
// energy; with dipole_flag writes dipole[0..11] and tm[0..53] for type 1
// (the caller zeroes them first).  phi = atan2(sin_phi, cos_phi) of the
// reference; the cosine series need only cos phi and sin phi, so types 0
// and 1 take them from the same two dot products without a trigonometric
// call (the improper, type 2, uses phi itself).
__device__ __forceinline__ void dihedral_term(V3 pa, V3 pb, V3 pc, V3 pd, const float* cf,
                                              const float* trig, int ty, int last,
                                              int dipole_flag, const Box& bx, V3 (&F)[4],
                                              float& e_out, float* dip, float* tmx) {
    const V3 fv = min_image(pa - pb, bx);
    const V3 g = min_image(pb - pc, bx);
    const V3 h = min_image(pd - pc, bx);
    const V3 v = cross(fv, g), w = cross(h, g);
    const float v_sq = dot(v, v), w_sq = dot(w, w);
    const float g_norm = norm(g);
    const float cos_phi = dot(v, w);
    const float sin_phi = dot(w, fv) * g_norm;
    const float f_dot_g = dot(fv, g), h_dot_g = dot(h, g);
    float e = 0.0f, df_dih = 0.0f;
    F[0] = F[1] = F[2] = F[3] = v3(0.f, 0.f, 0.f);
    if (ty == 0 || ty == 1) {
        const float rho2 = fmaf(cos_phi, cos_phi, sin_phi * sin_phi);
        float cphi = 1.0f, sphi = 0.0f;  // atan2(0, 0) = 0
        if (rho2 > 0.0f) {
            const float inv = 1.0f / sqrtf(rho2);
            cphi = cos_phi * inv;
            sphi = sin_phi * inv;
        }
        float C[5], S[5];
        multiples(cphi, sphi, C, S);
        cosine_series(cf, trig, trig + 15, C, S, e, df_dih);
        bool nz_c = false, nz_d = false;
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            nz_c |= cf[10 + q] != 0.0f;
            nz_d |= cf[15 + q] != 0.0f;
        }
        if (nz_c && nz_d) cosine_series(cf + 10, trig + 5, trig + 20, C, S, e, df_dih);
        if (ty == 1) {
            float e_cbt, df_cbt;
            V3 fa, fb, fc, fd;
            reconstruct(fv, pb, -g, bx, cf + 20, trig + 10, trig + 25, cphi, sphi, C, S,
                        dipole_flag, e_cbt, df_cbt, fa, fb, fc, dip, tmx);
            e += e_cbt;
            df_dih += df_cbt;
            F[0] = F[0] - fa;
            F[1] = F[1] - fb;
            F[2] = F[2] - fc;
            if (last == 1) {
                reconstruct(g, pc, h, bx, cf + 20, trig + 10, trig + 25, cphi, sphi, C, S,
                            dipole_flag, e_cbt, df_cbt, fb, fc, fd, dip ? dip + 6 : nullptr,
                            tmx ? tmx + 27 : nullptr);
                e += e_cbt;
                df_dih += df_cbt;
                F[1] = F[1] - fb;
                F[2] = F[2] - fc;
                F[3] = F[3] - fd;
            }
        }
    }
    if (ty == 2) {
        const float phi = atan2f(sin_phi, cos_phi);
        const float eq = cf[0], kc = cf[1];
        df_dih = kc * (phi - eq);
        e += 0.5f * kc * (phi - eq) * (phi - eq);
    }
    const V3 sc = (f_dot_g / (v_sq * g_norm)) * v - (h_dot_g / (w_sq * g_norm)) * w;
    const V3 fa = (-df_dih * g_norm / v_sq) * v;
    const V3 fd = (df_dih * g_norm / w_sq) * w;
    F[0] = F[0] + fa;
    F[1] = F[1] + (df_dih * sc - fa);
    F[2] = F[2] + (-df_dih * sc - fd);
    F[3] = F[3] + fd;
    e_out = e;
}

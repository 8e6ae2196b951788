// Forward-mode (dual number) FP32 arithmetic for directional derivatives of
// the bonded forces: a Dual carries a value and its derivative along one
// direction of the positions.  The bonded forces are minus the gradient of an
// energy, so their Jacobian is symmetric and the directional derivative along
// a cotangent lambda is also the vector-Jacobian product needed by reverse
// mode (a Hessian-vector product of the bonded energy).
#pragma once

#include "hpf_terms.cuh"

struct Dual {
    float v, t;
};

__device__ __forceinline__ Dual dual(float v, float t) { return Dual{v, t}; }
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return dual(a.v + b.v, a.t + b.t); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return dual(a.v - b.v, a.t - b.t); }
__device__ __forceinline__ Dual operator-(Dual a) { return dual(-a.v, -a.t); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) {
    return dual(a.v * b.v, fmaf(a.t, b.v, a.v * b.t));
}
__device__ __forceinline__ Dual operator*(float s, Dual a) { return dual(s * a.v, s * a.t); }
__device__ __forceinline__ Dual operator+(Dual a, float s) { return dual(a.v + s, a.t); }
__device__ __forceinline__ Dual operator-(Dual a, float s) { return dual(a.v - s, a.t); }
__device__ __forceinline__ Dual operator*(Dual a, float s) { return dual(a.v * s, a.t * s); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const float q = a.v / b.v;
    return dual(q, (a.t - q * b.t) / b.v);
}
__device__ __forceinline__ Dual operator/(float s, Dual b) {
    const float q = s / b.v;
    return dual(q, -q * b.t / b.v);
}
__device__ __forceinline__ Dual dsqrt(Dual a) {
    const float r = sqrtf(a.v);
    return dual(r, r > 0.0f ? 0.5f * a.t / r : 0.0f);
}
// |a| < 1
__device__ __forceinline__ Dual dacos(Dual a) {
    return dual(acosf(a.v), -a.t * rsqrtf(1.0f - a.v * a.v));
}
__device__ __forceinline__ Dual drsqrt(Dual a) {
    const float r = rsqrtf(a.v);
    return dual(r, -0.5f * r * r * r * a.t);
}
__device__ __forceinline__ Dual datan2(Dual y, Dual x) {
    const float den = fmaf(x.v, x.v, y.v * y.v);
    return dual(atan2f(y.v, x.v), (x.v * y.t - y.v * x.t) / den);
}

struct DV3 {
    Dual x, y, z;
};

__device__ __forceinline__ DV3 dv3(V3 v, V3 t) { return DV3{dual(v.x, t.x), dual(v.y, t.y), dual(v.z, t.z)}; }
__device__ __forceinline__ DV3 operator+(DV3 a, DV3 b) { return DV3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ DV3 operator-(DV3 a, DV3 b) { return DV3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ DV3 operator*(Dual s, DV3 a) { return DV3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ Dual ddot(DV3 a, DV3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ DV3 dcross(DV3 a, DV3 b) {
    return DV3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ DV3 operator-(DV3 a) { return DV3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 tangent(DV3 a) { return v3(a.x.t, a.y.t, a.z.t); }

// Directional derivative of bond_term's force on b (force on a: minus it),
// for the displacement directions la, lb of the two beads.
__device__ __forceinline__ V3 bond_force_tangent(V3 pa, V3 pb, V3 la, V3 lb, float r0, float k,
                                                 const Box& bx) {
    const DV3 rab = dv3(min_image(pb - pa, bx), lb - la);  // the image shift is constant
    const Dual d2 = ddot(rab, rab);
    const Dual ir = drsqrt(d2);
    const Dual dr = d2 * ir - dual(r0, 0.0f);
    return tangent((-k * dr * ir) * rab);
}

// Directional derivatives of angle_term's gradients ga (on a) and gc (on c);
// the forces are -ga on a, -gc on c, ga + gc on b.  Returns false where the
// triple is collinear (skipped, as in angle_term).
__device__ __forceinline__ bool angle_grad_tangent(V3 pa, V3 pb, V3 pc, V3 la, V3 lb, V3 lc,
                                                   float t0, float k, const Box& bx, V3& dga,
                                                   V3& dgc) {
    const DV3 ra = dv3(min_image(pa - pb, bx), la - lb);
    const DV3 rc = dv3(min_image(pc - pb, bx), lc - lb);
    const Dual ia = drsqrt(ddot(ra, ra)), ic = drsqrt(ddot(rc, rc));
    const DV3 ea = ia * ra, ec = ic * rc;
    const Dual cosphi = ddot(ea, ec);
    const DV3 cr = dcross(ea, ec);
    const Dual s2 = ddot(cr, cr);
    if (!(s2.v > 0.0f)) return false;
    const Dual is = drsqrt(s2);
    const Dual sinphi = s2 * is;
    const Dual theta = datan2(sinphi, cosphi);
    const Dual ff = k * (theta - dual(t0, 0.0f));
    dga = tangent((-ff * ia * is) * (ec - cosphi * ea));
    dgc = tangent((-ff * ic * is) * (ea - cosphi * ec));
    return true;
}

// ---- four-body term (compute_dihedral_forces.f90:61-134 and the bending
// part of dipole_reconstruction.f90:50-106), forward mode ----

// sum_n -n c_n sin(n phi - d_n) with cos phi, sin phi as duals (the phases
// cd, sd constant)
__device__ __forceinline__ Dual dcosine_series_de(const float* cn, const float* cd,
                                                  const float* sd, const Dual (&C)[5],
                                                  const Dual (&S)[5]) {
    Dual de = dual(0.0f, 0.0f);
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const Dual sn = S[i] * cd[i] - C[i] * sd[i];
        de = de + sn * (-(float)i * cn[i]);
    }
    return de;
}
__device__ __forceinline__ Dual dcosine_series_e(const float* cn, const float* cd,
                                                 const float* sd, const Dual (&C)[5],
                                                 const Dual (&S)[5]) {
    Dual e = dual(0.0f, 0.0f);
#pragma unroll
    for (int i = 0; i < 5; ++i) e = e + (C[i] * cd[i] + S[i] * sd[i] + 1.0f) * cn[i];
    return e;
}

// CBT bending of the angle (rab, rcb) at its middle bead, as reconstruct
// (hpf_terms.cuh) without the dipoles: adds minus the positive gradients to
// the forces on the angle's beads (Fa, Fb, Fc) and returns dE/dphi.
__device__ __forceinline__ Dual dreconstruct(DV3 rab, DV3 rcb, const float* c_k, const float* cd_k,
                                             const float* sd_k, Dual cphi, Dual sphi,
                                             const Dual (&C)[5], const Dual (&S)[5], DV3& Fa,
                                             DV3& Fb, DV3& Fc) {
    constexpr float c785 = 7.073882506e-01f, s785 = 7.068251997e-01f;  // cos, sin of 0.785f
    const Dual gamma_0 = (cphi * c785 + sphi * s785) * (-0.227f) + 1.85f;
    const Dual dg = (sphi * c785 - cphi * s785) * 0.227f;
    const Dual k = dcosine_series_e(c_k, cd_k, sd_k, C, S);
    const Dual dk = dcosine_series_de(c_k, cd_k, sd_k, C, S);
    const Dual norm_a = dsqrt(ddot(rab, rab)), norm_c = dsqrt(ddot(rcb, rcb));
    const DV3 w = (1.0f / norm_a) * rab, v = (1.0f / norm_c) * rcb;
    const Dual cos_gamma = ddot(w, v);
    if (!(cos_gamma.v * cos_gamma.v < 1.0f)) return dual(0.0f, 0.0f);
    const Dual gamm = dacos(cos_gamma);
    Dual sin_gamma = dsqrt(dual(1.0f, 0.0f) - cos_gamma * cos_gamma);
    if (sin_gamma.v < 0.1f) sin_gamma = dual(0.1f, 0.0f);
    const DV3 fa = (-1.0f / (norm_a * sin_gamma)) * (v - cos_gamma * w);
    const DV3 fc = (-1.0f / (norm_c * sin_gamma)) * (w - cos_gamma * v);
    const DV3 fb = -(fa + fc);
    const Dual df_ang = k * (gamm - gamma_0);
    const Dual var_sq = (gamm - gamma_0) * (gamm - gamma_0);
    Fa = Fa - df_ang * fa;
    Fb = Fb - df_ang * fb;
    Fc = Fc - df_ang * fc;
    return dk * var_sq * 0.5f - df_ang * dg;
}

// Directional derivatives dF[0..3] of dihedral_term's forces on a, b, c, d
// along the displacements la..ld (no dipoles).
__device__ __forceinline__ void dihedral_force_tangent(V3 pa, V3 pb, V3 pc, V3 pd, V3 la, V3 lb,
                                                       V3 lc, V3 ld, const float* cf,
                                                       const float* trig, int ty, int last,
                                                       const Box& bx, V3 (&dF)[4]) {
    const DV3 fv = dv3(min_image(pa - pb, bx), la - lb);  // image shifts are constant
    const DV3 g = dv3(min_image(pb - pc, bx), lb - lc);
    const DV3 h = dv3(min_image(pd - pc, bx), ld - lc);
    const DV3 v = dcross(fv, g), w = dcross(h, g);
    const Dual v_sq = ddot(v, v), w_sq = ddot(w, w);
    const Dual g_norm = dsqrt(ddot(g, g));
    const Dual cos_phi = ddot(v, w);
    const Dual sin_phi = ddot(w, fv) * g_norm;
    const Dual f_dot_g = ddot(fv, g), h_dot_g = ddot(h, g);
    const Dual zero = dual(0.0f, 0.0f);
    DV3 F[4] = {{zero, zero, zero}, {zero, zero, zero}, {zero, zero, zero}, {zero, zero, zero}};
    Dual df_dih = zero;
    if (ty == 0 || ty == 1) {
        const Dual rho2 = cos_phi * cos_phi + sin_phi * sin_phi;
        Dual cphi = dual(1.0f, 0.0f), sphi = zero;
        if (rho2.v > 0.0f) {
            const Dual inv = 1.0f / dsqrt(rho2);
            cphi = cos_phi * inv;
            sphi = sin_phi * inv;
        }
        Dual C[5], S[5];
        C[0] = dual(1.0f, 0.0f);
        S[0] = zero;
#pragma unroll
        for (int q = 1; q < 5; ++q) {
            C[q] = C[q - 1] * cphi - S[q - 1] * sphi;
            S[q] = S[q - 1] * cphi + C[q - 1] * sphi;
        }
        df_dih = dcosine_series_de(cf, trig, trig + 15, C, S);
        bool nz_c = false, nz_d = false;
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            nz_c |= cf[10 + q] != 0.0f;
            nz_d |= cf[15 + q] != 0.0f;
        }
        if (nz_c && nz_d) df_dih = df_dih + dcosine_series_de(cf + 10, trig + 5, trig + 20, C, S);
        if (ty == 1) {
            df_dih = df_dih + dreconstruct(fv, -g, cf + 20, trig + 10, trig + 25, cphi, sphi, C, S,
                                           F[0], F[1], F[2]);
            if (last == 1)
                df_dih = df_dih + dreconstruct(g, h, cf + 20, trig + 10, trig + 25, cphi, sphi, C,
                                               S, F[1], F[2], F[3]);
        }
    }
    if (ty == 2) {
        const Dual phi = datan2(sin_phi, cos_phi);
        df_dih = (phi - cf[0]) * cf[1];
    }
    const DV3 sc = (f_dot_g / (v_sq * g_norm)) * v - (h_dot_g / (w_sq * g_norm)) * w;
    const DV3 fa = (-df_dih * g_norm / v_sq) * v;
    const DV3 fd = (df_dih * g_norm / w_sq) * w;
    dF[0] = tangent(F[0] + fa);
    dF[1] = tangent(F[1] + (df_dih * sc - fa));
    dF[2] = tangent(F[2] + (-df_dih * sc - fd));
    dF[3] = tangent(F[3] + fd);
}

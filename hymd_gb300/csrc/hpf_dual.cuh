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

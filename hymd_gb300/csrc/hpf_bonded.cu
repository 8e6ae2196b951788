// Bonded forces of HyMD on GB300, f2py calling form: harmonic bonds, harmonic
// angles, cosine-series / combined bending-torsion / improper dihedrals with
// the peptide dipole reconstruction, and the redistribution of dipole forces.
//
// Reference behaviour (paths inside the HyMD project):
//   cbf   hymd/compute_bond_forces.f90:1-61
//   caf   hymd/compute_angle_forces.f90:1-93
//   cdf   hymd/compute_dihedral_forces.f90:1-137
//   dipole_forces_redistribution hymd/force.py:855-877
//
// One thread per term (the per-term arithmetic lives in hpf_terms.cuh and is
// shared with the fused rRESPA kernel).  Energies and virials are summed in
// FP64 by a deterministic grid reduction; forces are accumulated with FP32
// atomics into the zeroed force array.
#include "hpf_dual.cuh"
#include "hpf_internal.cuh"
#include "hpf_terms.cuh"

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ V3 load3(const float* r, int i) {
    return v3(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
}

__device__ __forceinline__ void add3(float* f, int i, V3 v) {
    atomicAdd(f + 3 * i, v.x);
    atomicAdd(f + 3 * i + 1, v.y);
    atomicAdd(f + 3 * i + 2, v.z);
}

__device__ __forceinline__ bool in_range(int i, int64_t n) { return i >= 0 && (int64_t)i < n; }

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
        float e;
        V3 vir;
        const V3 fa = bond_term(load3(r, ia), load3(r, ib), r0[i], kk[i], bx, e, vir);
        add3(f, ia, -fa);
        add3(f, ib, fa);
        acc[0] += (double)e;
        acc[1] += (double)vir.x;
        acc[2] += (double)vir.y;
        acc[3] += (double)vir.z;
    }
    grid_reduce_store<4>(acc, ws_partials(out), ws_ticket(out), out, false);
}

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
        V3 ga, gc, vir;
        float e;
        if (!angle_term(load3(r, ia), load3(r, ib), load3(r, ic), t0[i], kk[i], bx, ga, gc, e, vir))
            continue;
        add3(f, ia, -ga);
        add3(f, ic, -gc);
        add3(f, ib, ga + gc);
        acc[0] += (double)e;
        acc[1] += (double)vir.x;
        acc[2] += (double)vir.y;
        acc[3] += (double)vir.z;
    }
    grid_reduce_store<4>(acc, ws_partials(out), ws_ticket(out), out, false);
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
        const int idx[4] = {a[i], b[i], c[i], d[i]};
        if (!in_range(idx[0], n) || !in_range(idx[1], n) || !in_range(idx[2], n) ||
            !in_range(idx[3], n)) {
            hpf_flag(err, HPF_ERR_INDEX);
            continue;
        }
        V3 F[4];
        float e;
        float trig[30];
        dih_phase_trig(coeff + 30 * i, trig);
        dihedral_term(load3(r, idx[0]), load3(r, idx[1]), load3(r, idx[2]), load3(r, idx[3]),
                      coeff + 30 * i, trig, dtype[i], last[i], dipole_flag, bx, F, e, dip, tmx);
#pragma unroll
        for (int q = 0; q < 4; ++q) add3(force, idx[q], F[q]);
        acc[0] += (double)e;
    }
    grid_reduce_store<1>(acc, ws_partials(out), ws_ticket(out), out, false);
}

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
            // beads (a, b, c) for the first dipole pair, (b, c, d) for the last angle
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


// Directional derivative of the bond and angle forces along lambda (the
// Hessian-vector product of the bonded energy, with a minus sign), summed
// into out with FP32 atomics.
__global__ void k_bonds_hvp(float* __restrict__ out, const float* __restrict__ r,
                            const float* __restrict__ lam, int64_t n,
                            const double* __restrict__ box, const int32_t* __restrict__ a,
                            const int32_t* __restrict__ b, const float* __restrict__ r0,
                            const float* __restrict__ k, int64_t nb, int* err) {
    const Box bx = load_box(box);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nb;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int ia = a[t], ib = b[t];
        if (!in_range(ia, n) || !in_range(ib, n)) {
            hpf_flag(err, HPF_ERR_INDEX);
            continue;
        }
        const V3 dfb = bond_force_tangent(load3(r, ia), load3(r, ib), load3(lam, ia),
                                          load3(lam, ib), r0[t], k[t], bx);
        add3(out, ia, -dfb);
        add3(out, ib, dfb);
    }
}

__global__ void k_angles_hvp(float* __restrict__ out, const float* __restrict__ r,
                             const float* __restrict__ lam, int64_t n,
                             const double* __restrict__ box, const int32_t* __restrict__ a,
                             const int32_t* __restrict__ b, const int32_t* __restrict__ c,
                             const float* __restrict__ t0, const float* __restrict__ k,
                             int64_t na, int* err) {
    const Box bx = load_box(box);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < na;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int ia = a[t], ib = b[t], ic = c[t];
        if (!in_range(ia, n) || !in_range(ib, n) || !in_range(ic, n)) {
            hpf_flag(err, HPF_ERR_INDEX);
            continue;
        }
        V3 dga, dgc;
        if (!angle_grad_tangent(load3(r, ia), load3(r, ib), load3(r, ic), load3(lam, ia),
                                load3(lam, ib), load3(lam, ic), t0[t], k[t], bx, dga, dgc))
            continue;
        add3(out, ia, -dga);
        add3(out, ic, -dgc);
        add3(out, ib, dga + dgc);
    }
}

__global__ void k_dihedrals_hvp(float* __restrict__ out, const float* __restrict__ r,
                                const float* __restrict__ lam, int64_t n,
                                const double* __restrict__ box, const int32_t* __restrict__ a,
                                const int32_t* __restrict__ b, const int32_t* __restrict__ c,
                                const int32_t* __restrict__ d, const float* __restrict__ coeff,
                                const int32_t* __restrict__ dtype,
                                const int32_t* __restrict__ last, int64_t nd, int* err) {
    const Box bx = load_box(box);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nd;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int idx[4] = {a[t], b[t], c[t], d[t]};
        if (!in_range(idx[0], n) || !in_range(idx[1], n) || !in_range(idx[2], n) ||
            !in_range(idx[3], n)) {
            hpf_flag(err, HPF_ERR_INDEX);
            continue;
        }
        float trig[30];
        dih_phase_trig(coeff + 30 * t, trig);
        V3 dF[4];
        dihedral_force_tangent(load3(r, idx[0]), load3(r, idx[1]), load3(r, idx[2]),
                               load3(r, idx[3]), load3(lam, idx[0]), load3(lam, idx[1]),
                               load3(lam, idx[2]), load3(lam, idx[3]), coeff + 30 * t, trig,
                               dtype[t], last[t], bx, dF);
#pragma unroll
        for (int q = 0; q < 4; ++q) add3(out, idx[q], dF[q]);
    }
}

}  // namespace

extern "C" {

int hpf_dihedral_hvp(float* out, const float* r, const float* lam, int64_t n, const double* box,
                     const int32_t* a, const int32_t* b, const int32_t* c, const int32_t* d,
                     const float* coeff, const int32_t* dtype, const int32_t* last, int64_t nd,
                     int* d_err, void* stream) {
    if (!out || !r || !lam || !box || n < 0 || nd < 0 ||
        (nd > 0 && (!a || !b || !c || !d || !coeff || !dtype || !last)))
        return HPF_ERR_ARG;
    if (nd == 0) return HPF_OK;
    k_dihedrals_hvp<<<grid_for(nd), kThreads, 0, as_stream(stream)>>>(
        out, r, lam, n, box, a, b, c, d, coeff, dtype, last, nd, d_err);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

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

int hpf_bonded_hvp(float* out, const float* r, const float* lam, int64_t n, const double* box,
                   const int32_t* ba, const int32_t* bb, const float* br0, const float* bk,
                   int64_t nb, const int32_t* aa, const int32_t* ab, const int32_t* ac,
                   const float* at0, const float* ak, int64_t na, int* d_err, void* stream) {
    if (!out || !r || !lam || !box || n < 0 || nb < 0 || na < 0 ||
        (nb > 0 && (!ba || !bb || !br0 || !bk)) || (na > 0 && (!aa || !ab || !ac || !at0 || !ak)))
        return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    HPF_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * 3 * (size_t)n, st));
    if (nb > 0) {
        k_bonds_hvp<<<grid_for(nb), kThreads, 0, st>>>(out, r, lam, n, box, ba, bb, br0, bk, nb,
                                                       d_err);
        HPF_LAUNCH_CHECK();
    }
    if (na > 0) {
        k_angles_hvp<<<grid_for(na), kThreads, 0, st>>>(out, r, lam, n, box, aa, ab, ac, at0, ak,
                                                        na, d_err);
        HPF_LAUNCH_CHECK();
    }
    return HPF_OK;
}

}  // extern "C"

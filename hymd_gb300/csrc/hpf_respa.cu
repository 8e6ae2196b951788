// Fused rRESPA inner loop of HyMD on GB300 (hymd/main.py:802-887).
//
// Bonded terms never couple different molecules, so the whole inner loop --
// respa_inner x (half kick, drift, wrap, bonded forces, half kick) -- needs no
// grid-wide synchronisation if a group of threads owns whole molecules.  The
// planner (host C++) finds the molecules as connected components of the
// bonded terms, packs them into groups of at most `max_group_beads` beads and
// rewrites every term with group-local bead indices.  One launch then:
//   * molecule groups: stage positions, velocities, bonded forces and the
//     group's topology in shared memory, apply the first outer half kick with
//     the slow forces, run all inner steps on chip, write back.  Groups of up
//     to 64 beads are run by one warp each (phases separated by __syncwarp),
//     larger ones by a whole CTA (__syncthreads);
//   * free beads (in no bonded term): per thread, the outer kick and
//     respa_inner drift/wrap steps (their bonded force is zero).
// Forces are accumulated without atomics: every term writes its force
// vectors into its own shared-memory slots, then every bead adds the slots
// that touch it in a fixed order (incidence lists built by the planner), so
// the bonded forces are bit-deterministic.
// Energies and virials of the last inner step (the ones the reference keeps,
// main.py:964-973) and sum v^2 are written as block partials and summed by a
// one-block finish kernel, which can also run the isotropic SCR barostat
// (hymd/barostat_scr.py:34-132) there, since the barostat follows the inner
// loop (main.py:889-963).
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "hpf_internal.cuh"
#include "hpf_terms.cuh"

struct hpf_respa_plan {
    int64_t n_beads;
    int n_groups;        // molecule groups
    int n_bonded;        // beads in groups (entries of bead_ids)
    int n_free;
    int n_free_blocks;
    int warp_mode;       // 1: one warp per group, 0: one CTA per group
    int has_dih;
    // per-group maxima (shared-memory layout)
    int mx_beads, mx_slots, mx_inc, mx_bonds, mx_angles;
    size_t smem_group;   // bytes per group
    size_t smem;         // dynamic shared memory per block
    // device arrays
    int* grp_bead;    // [n_groups+1]
    int* bead_ids;    // bonded beads, group-major
    int* bead_inc;    // [n_bonded_beads+1] incidence list starts (group-major beads)
    int* inc_list;    // (slot << 1) | negative, slot local to the group
    int* grp_bond;    // [n_groups+1]
    int* bond_ij;     // local indices, i | j << 16
    float2* bond_p;   // (r0, k)
    int* grp_ang;
    int2* ang_ijk;    // (i | j << 16, k)
    float2* ang_p;    // (t0, k)
    int* grp_dih;
    short4* dih_ijkl;
    float* dih_coeff;  // 30 per term
    float* dih_trig;   // 30 per term: cos / sin of the phase rows (dih_phase_trig)
    int2* dih_tl;      // (type, last)
    int* dih_gid;      // global dihedral index (dipole / transfer rows)
    int* free_ids;
    double* partials;   // [kOut][grid] block partials (float2 hi/lo per slot)
    // second stream of the split launch (free beads beside the groups) and
    // its fork / join events
    cudaStream_t free_stream;
    cudaEvent_t free_fork, free_join;
};

namespace {

constexpr int kThreads = 128;  // 4 warps
constexpr int kWarps = kThreads / 32;
constexpr int kMaxSlow = 4;
constexpr int kOut = 10;  // E_bond, pr_bond[3], E_angle, pr_angle[3], E_dihedral, sum v^2
// Groups of up to this many beads run one per warp (about two beads and two
// terms of each kind per lane); larger ones one per CTA, so that a long chain
// gets one thread per bead and per term instead of a serial loop per lane.
constexpr int kWarpMaxBeads = 64;

struct SlowForces {
    const float* f[kMaxSlow];
    int n;
};

// Optional barostat run by the finish kernel (all inner steps are done then).
struct BaroFuse {
    int on;
    HpfScrArgs a;
    const double* field;
    const double* randoms;
    int* counter;
    BoxState* bs;
    const Functional* fun;
    double* state;
};

// np.mod(x, L), L > 0.  A drift moves a bead far less than a box length, so
// x lies in (-L, 2L): then x - L (Sterbenz, exact) or x + L equals fmod's
// result; anything else takes fmodf.
__device__ __forceinline__ float wrapf(float x, float L) {
    if (x >= 0.0f && x < L) return x;
    if (x >= L && x < 2.0f * L) return x - L;
    if (x < 0.0f && x > -L) return x + L;
    float m = fmodf(x, L);
    if (m < 0.0f) m += L;
    return m;
}

struct WarpSync {
    __device__ __forceinline__ void operator()() const { __syncwarp(); }
};
struct CtaSync {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

// Shared-memory layout of one group (offsets in bytes, 16-byte aligned).
// Bead positions, velocities, forces and the term force slots are float4
// (x, y, z, unused): one 128-bit shared-memory access per vector.
struct GroupSmem {
    float2 *bond_p, *ang_p;
    int2* ang_ijk;
    float4 *rs, *vs, *fs, *slot;
    int *bond_ij, *inc_start, *inc;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline size_t group_smem_bytes(int nb, int ns, int ni, int nbd, int na) {
    size_t o = 0;
    o += align16(sizeof(float2) * nbd);  // bond_p
    o += align16(sizeof(float2) * na);   // ang_p
    o += align16(sizeof(int2) * na);     // ang_ijk
    o += align16(sizeof(float4) * 3 * nb);
    o += align16(sizeof(float4) * ns);
    o += align16(sizeof(int) * nbd);
    o += align16(sizeof(int) * (nb + 1));
    o += align16(sizeof(int) * ni);
    return o;
}

__device__ __forceinline__ GroupSmem carve(char* base, const hpf_respa_plan& p) {
    GroupSmem g;
    size_t o = 0;
    g.bond_p = reinterpret_cast<float2*>(base + o);
    o += align16(sizeof(float2) * p.mx_bonds);
    g.ang_p = reinterpret_cast<float2*>(base + o);
    o += align16(sizeof(float2) * p.mx_angles);
    g.ang_ijk = reinterpret_cast<int2*>(base + o);
    o += align16(sizeof(int2) * p.mx_angles);
    g.rs = reinterpret_cast<float4*>(base + o);
    g.vs = g.rs + p.mx_beads;
    g.fs = g.rs + 2 * p.mx_beads;
    o += align16(sizeof(float4) * 3 * p.mx_beads);
    g.slot = reinterpret_cast<float4*>(base + o);
    o += align16(sizeof(float4) * p.mx_slots);
    g.bond_ij = reinterpret_cast<int*>(base + o);
    o += align16(sizeof(int) * p.mx_bonds);
    g.inc_start = reinterpret_cast<int*>(base + o);
    o += align16(sizeof(int) * (p.mx_beads + 1));
    g.inc = reinterpret_cast<int*>(base + o);
    return g;
}

__device__ __forceinline__ void put3(float4* s, int slot, V3 v) {
    s[slot] = make_float4(v.x, v.y, v.z, 0.0f);
}

__device__ __forceinline__ V3 get3(const float4* s, int i) {
    const float4 q = s[i];
    return v3(q.x, q.y, q.z);
}

__device__ __forceinline__ float comp(const float4& q, int d) {
    return d == 0 ? q.x : (d == 1 ? q.y : q.z);
}

// The write-back's deposit of a group bead, out of line: the group kernels
// run near their register limit in the term loop, and the deposit's
// addresses and weights would add to it.
__device__ __noinline__ void paint_group_bead(PaintFuse pf, int64_t bead, float x, float y,
                                              float z) {
    paint_bead(pf, cic_mesh(pf.bs), bead, x, y, z);
}

// Group-local work shared by the warp and CTA variants.  `lane`/`width`
// enumerate the threads of the group; `sync()` separates the phases.  A
// bead is always handled by the same lane, so the gather of its forces and
// its next kick need no barrier in between.
template <bool DIH, bool PAINT, typename Sync>
__device__ __forceinline__ void run_group(const hpf_respa_plan& p, int grp, int lane, int width,
                                          char* smem_base, float* __restrict__ r,
                                          float* __restrict__ v, float* __restrict__ fb,
                                          const SlowForces& slow, float mass, float h_out,
                                          float hdt, float dt, int respa, const Box& bx,
                                          float* __restrict__ dipoles,
                                          float* __restrict__ transfer, float (&acc)[kOut],
                                          Sync sync, bool forces_only, const PaintFuse& pf) {
    // forces_only: bonded forces (and energies) at the current positions
    // only -- no kicks, no drift, v and r untouched (respa is 1 then)
    const GroupSmem s = carve(smem_base, p);
    const int s0 = p.grp_bead[grp], nb = p.grp_bead[grp + 1] - s0;
    const int b0 = p.grp_bond[grp], nbd = p.grp_bond[grp + 1] - b0;
    const int a0 = p.grp_ang[grp], na = p.grp_ang[grp + 1] - a0;
    const int d0 = DIH ? p.grp_dih[grp] : 0, nd = DIH ? p.grp_dih[grp + 1] - d0 : 0;
    const int i0 = p.bead_inc[s0];
    const float inv_m = 1.0f / mass;
    // stage the group: beads (with the first outer half kick), topology
    for (int e = lane; e < 3 * nb; e += width) {
        const int i = e / 3, d = e - 3 * i;
        const int64_t g = 3 * (int64_t)p.bead_ids[s0 + i] + d;
        float x = forces_only ? 0.0f : v[g];
#pragma unroll
        for (int q = 0; q < kMaxSlow; ++q)
            if (q < slow.n) x = x + h_out * div_m(slow.f[q][g], mass, inv_m);
        reinterpret_cast<float*>(s.vs + i)[d] = x;
        reinterpret_cast<float*>(s.rs + i)[d] = r[g];
        reinterpret_cast<float*>(s.fs + i)[d] = fb[g];
    }
    for (int t = lane; t < nbd; t += width) {
        s.bond_ij[t] = p.bond_ij[b0 + t];
        s.bond_p[t] = p.bond_p[b0 + t];
    }
    for (int t = lane; t < na; t += width) {
        s.ang_ijk[t] = p.ang_ijk[a0 + t];
        s.ang_p[t] = p.ang_p[a0 + t];
    }
    for (int i = lane; i <= nb; i += width) s.inc_start[i] = p.bead_inc[s0 + i] - i0;
    const int ninc = p.bead_inc[s0 + nb] - i0;
    for (int t = lane; t < ninc; t += width) s.inc[t] = p.inc_list[i0 + t];
    sync();
    for (int it = 0; it <= respa; ++it) {
        const bool last_it = it == respa - 1;
        // per bead: gather the bonded force of the previous inner step (in
        // the fixed incidence order), closing half kick of that step; then,
        // unless all steps are done, the opening half kick, drift and wrap
        for (int i = lane; i < nb; i += width) {
            float4 F;
            if (it == 0) {
                F = s.fs[i];
            } else {
                // signed sum in the fixed incidence order; fmaf(-1, x, F) is
                // the exactly rounded F - x, so no branch on the sign
                F = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                for (int q = s.inc_start[i]; q < s.inc_start[i + 1]; ++q) {
                    const int en = s.inc[q];
                    const float4 sl = s.slot[en >> 1];
                    const float sg = (en & 1) ? -1.0f : 1.0f;
                    F.x = fmaf(sg, sl.x, F.x);
                    F.y = fmaf(sg, sl.y, F.y);
                    F.z = fmaf(sg, sl.z, F.z);
                }
                s.fs[i] = F;
            }
            if (forces_only) continue;
            float4 rv = s.rs[i], vv = s.vs[i];
            float xr[3] = {rv.x, rv.y, rv.z}, xv[3] = {vv.x, vv.y, vv.z};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const float a = div_m(comp(F, d), mass, inv_m);
                float x = xv[d];
                if (it > 0) x = x + hdt * a;
                if (it < respa) {
                    x = x + hdt * a;
                    xr[d] = wrapf(xr[d] + dt * x, bx.L[d]);
                }
                xv[d] = x;
            }
            s.vs[i] = make_float4(xv[0], xv[1], xv[2], 0.0f);
            s.rs[i] = make_float4(xr[0], xr[1], xr[2], 0.0f);
        }
        if (it == respa) break;
        sync();
        // Term work in chunks of 32 terms of one kind, dealt round-robin to
        // the group's warps with the dihedrals (the longest) first: with a
        // whole CTA on a chain no lane computes a dihedral, an angle and a
        // bond one after the other.  A warp takes its chunks in order; each
        // term still writes only its own slots.
        const int wid = lane >> 5, nw = width >> 5, l32 = lane & 31;
        const int cd = DIH ? (nd + 31) >> 5 : 0, ca = (na + 31) >> 5, cb = (nbd + 31) >> 5;
        for (int task = wid; task < cd + ca + cb; task += nw) {
            if (DIH && task < cd) {
                const int t = (task << 5) + l32;
                if (t >= nd) continue;
                const short4 q = p.dih_ijkl[d0 + t];
                const int2 tl = p.dih_tl[d0 + t];
                const V3 p0 = get3(s.rs, q.x), p1 = get3(s.rs, q.y);
                const V3 p2 = get3(s.rs, q.z), p3 = get3(s.rs, q.w);
                float* dip = nullptr;
                float* tmx = nullptr;
                if (last_it && dipoles) {
                    const int64_t gd = p.dih_gid[d0 + t];
                    dip = dipoles + 12 * gd;
                    tmx = transfer + 54 * gd;
                    for (int j = 0; j < 12; ++j) dip[j] = 0.0f;
                    for (int j = 0; j < 54; ++j) tmx[j] = 0.0f;
                }
                V3 F[4];
                float e;
                const int64_t c30 = 30 * (int64_t)(d0 + t);
                dihedral_term(p0, p1, p2, p3, p.dih_coeff + c30, p.dih_trig + c30, tl.x, tl.y,
                              (last_it && dipoles) ? 1 : 0, bx, F, e, dip, tmx);
                const int sl = nbd + 2 * na + t;
#pragma unroll
                for (int j = 0; j < 4; ++j) put3(s.slot, sl + j * nd, F[j]);
                if (last_it) acc[8] += e;
            } else if (task < cd + ca) {
                const int t = ((task - cd) << 5) + l32;
                if (t >= na) continue;
                const int2 q = s.ang_ijk[t];
                const int ai = q.x & 0xffff, aj = q.x >> 16, ak = q.y;
                const float2 pr = s.ang_p[t];
                const V3 pa = get3(s.rs, ai);
                const V3 pb = get3(s.rs, aj);
                const V3 pc = get3(s.rs, ak);
                V3 ga, gc, vir;
                float e;
                if (!angle_term(pa, pb, pc, pr.x, pr.y, bx, ga, gc, e, vir)) {
                    ga = gc = v3(0.f, 0.f, 0.f);
                    e = 0.0f;
                    vir = ga;
                }
                put3(s.slot, nbd + t, ga);
                put3(s.slot, nbd + na + t, gc);
                if (last_it) {
                    acc[4] += e;
                    acc[5] += vir.x;
                    acc[6] += vir.y;
                    acc[7] += vir.z;
                }
            } else {
                const int t = ((task - cd - ca) << 5) + l32;
                if (t >= nbd) continue;
                const int ij = s.bond_ij[t];
                const int bi = ij & 0xffff, bj = ij >> 16;
                const float2 pr = s.bond_p[t];
                float e;
                V3 vir;
                const V3 pa = get3(s.rs, bi);
                const V3 pb = get3(s.rs, bj);
                put3(s.slot, t, bond_term(pa, pb, pr.x, pr.y, bx, e, vir));
                if (last_it) {
                    acc[0] += e;
                    acc[1] += vir.x;
                    acc[2] += vir.y;
                    acc[3] += vir.z;
                }
            }
        }
        sync();
    }
    // write back (each bead by the lane that owns it); with PAINT the bead is
    // deposited on the mesh at its final position
    for (int i = lane; i < nb; i += width) {
        const int64_t bead = p.bead_ids[s0 + i], g = 3 * bead;
        const float4 fq = s.fs[i];
        if (forces_only) {
            for (int d = 0; d < 3; ++d) fb[g + d] = comp(fq, d);
            continue;
        }
        const float4 vq = s.vs[i], rq = s.rs[i];
        for (int d = 0; d < 3; ++d) {
            const float x = comp(vq, d);
            v[g + d] = x;
            r[g + d] = comp(rq, d);
            fb[g + d] = comp(fq, d);
            acc[9] = fmaf(x, x, acc[9]);
        }
        if (PAINT) paint_group_bead(pf, bead, rq.x, rq.y, rq.z);
    }
}

template <bool PAINT>
__device__ __forceinline__ void free_beads(const hpf_respa_plan& p, int fblock, float* __restrict__ r,
                                           float* __restrict__ v, const SlowForces& slow,
                                           float mass, float h_out, float dt, int respa,
                                           const Box& bx, float (&acc)[kOut],
                                           const PaintFuse& pf) {
    const int stride = p.n_free_blocks * kThreads;
    const float inv_m = 1.0f / mass;
    CicMesh cm;
    if (PAINT) cm = cic_mesh(pf.bs);
    for (int j = fblock * kThreads + threadIdx.x; j < p.n_free; j += stride) {
        const int64_t bead = p.free_ids[j], g = 3 * bead;
        float yr[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            float x = v[g + d];
#pragma unroll
            for (int q = 0; q < kMaxSlow; ++q)
                if (q < slow.n) x = x + h_out * div_m(slow.f[q][g + d], mass, inv_m);
            float y = r[g + d];
            for (int it = 0; it < respa; ++it) y = wrapf(y + dt * x, bx.L[d]);
            v[g + d] = x;
            r[g + d] = y;
            yr[d] = y;
            acc[9] = fmaf(x, x, acc[9]);
        }
        // a free bead's position is final after its drift: deposit it now,
        // while the molecule groups are still integrating
        if (PAINT) paint_bead(pf, cm, bead, yr[0], yr[1], yr[2]);
    }
}

template <bool DIH, bool PAINT>
__global__ void __launch_bounds__(kThreads)
k_respa_warp(hpf_respa_plan p, float* __restrict__ r, float* __restrict__ v,
             float* __restrict__ fb, SlowForces slow, float mass, float h_out, float hdt, float dt,
             int respa, const double* __restrict__ box, float* __restrict__ dipoles,
             float* __restrict__ transfer, double* out, int forces_only, PaintFuse pf,
             unsigned int G) {
    extern __shared__ __align__(16) char smem[];
    const Box bx = load_box(box);
    float acc[kOut];
#pragma unroll
    for (int k = 0; k < kOut; ++k) acc[k] = 0.0f;
    const int n_grp_blocks = (p.n_groups + kWarps - 1) / kWarps;
    if ((int)blockIdx.x < n_grp_blocks) {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const int grp = blockIdx.x * kWarps + warp;
        if (grp < p.n_groups)
            run_group<DIH, PAINT>(p, grp, lane, 32, smem + (size_t)warp * p.smem_group, r, v, fb,
                                  slow, mass, h_out, hdt, dt, respa, bx, dipoles, transfer, acc,
                                  WarpSync(), forces_only != 0, pf);
    } else if (!forces_only) {
        free_beads<PAINT>(p, blockIdx.x - n_grp_blocks, r, v, slow, mass, h_out, dt, respa, bx,
                          acc, pf);
    }
    if (out) block_partials_f<kOut, kThreads>(acc, p.partials, G);
}

// Four blocks per SM: the chain CTAs share the SMs with the free-bead
// blocks, which need the occupancy to hide their global loads.
template <bool DIH, bool PAINT>
__global__ void __launch_bounds__(kThreads, 4)
k_respa_cta(hpf_respa_plan p, float* __restrict__ r, float* __restrict__ v,
            float* __restrict__ fb, SlowForces slow, float mass, float h_out, float hdt, float dt,
            int respa, const double* __restrict__ box, float* __restrict__ dipoles,
            float* __restrict__ transfer, double* out, int forces_only, PaintFuse pf,
            unsigned int G) {
    extern __shared__ __align__(16) char smem[];
    const Box bx = load_box(box);
    float acc[kOut];
#pragma unroll
    for (int k = 0; k < kOut; ++k) acc[k] = 0.0f;
    if ((int)blockIdx.x < p.n_groups) {
        run_group<DIH, PAINT>(p, blockIdx.x, threadIdx.x, kThreads, smem, r, v, fb, slow, mass,
                              h_out, hdt, dt, respa, bx, dipoles, transfer, acc, CtaSync(),
                              forces_only != 0, pf);
    } else if (!forces_only) {
        free_beads<PAINT>(p, blockIdx.x - p.n_groups, r, v, slow, mass, h_out, dt, respa, bx,
                          acc, pf);
    }
    if (out) block_partials_f<kOut, kThreads>(acc, p.partials, G);
}

// The free beads of a split launch, beside the group kernel (on a second
// stream): the free-bead blocks of k_respa_warp / k_respa_cta with the same
// beads per block, without the groups' dynamic shared memory, so that they
// fill the SMs around the group blocks; partials at slots slot0 + block, as
// in the single launch.
template <bool PAINT>
__global__ void __launch_bounds__(kThreads)
k_respa_free(hpf_respa_plan p, float* __restrict__ r, float* __restrict__ v, SlowForces slow,
             float mass, float h_out, float dt, int respa, const double* __restrict__ box,
             double* out, PaintFuse pf, unsigned int G, unsigned int slot0) {
    const Box bx = load_box(box);
    float acc[kOut];
#pragma unroll
    for (int k = 0; k < kOut; ++k) acc[k] = 0.0f;
    free_beads<PAINT>(p, blockIdx.x, r, v, slow, mass, h_out, dt, respa, bx, acc, pf);
    if (out) block_partials_f<kOut, kThreads>(acc, p.partials, G, slot0 + blockIdx.x);
}

// ids[k] = inv[ids[k]]: the plan's bead lists follow a permutation of the
// bead arrays (inv[old index] = new index); an index outside [0, n) is
// flagged and left as it was.
__global__ void k_remap_ids(int* __restrict__ ids, int64_t count, const int32_t* __restrict__ inv,
                            int64_t n, int* err) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int i = ids[k];
        if (i < 0 || i >= n) {
            if (err) atomicCAS(err, 0, HPF_ERR_INDEX);
            continue;
        }
        ids[k] = inv[i];
    }
}

// cos / sin of every dihedral's phase rows, once per plan (dih_phase_trig:
// the values the per-term kernel computes for itself).
__global__ void k_dih_trig(const float* __restrict__ coeff, float* __restrict__ trig, int64_t nd) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < nd) dih_phase_trig(coeff + 30 * i, trig + 30 * i);
}

// Sum of the block partials (fixed order) into out[0..kOut), then the
// barostat when coupled.  A separate one-block launch: a last-block reduction
// inside the main kernel (fence + ticket on every block, then a serial pass
// at the end) cost more than this launch.
//
// The pass is one latency chain, so it is kept short: every thread loads all
// its partials before adding (up to kFinishRounds x 256 blocks in one round
// trip), the sums stay in shared memory for the barostat, and one warp
// fetches the barostat's inputs into L1 while the partials are summed.
constexpr int kFinishThreads = 256;
constexpr int kFinishRounds = 6;

__device__ __forceinline__ void prefetch_l1(const void* p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

__global__ void __launch_bounds__(kFinishThreads)
k_respa_finish(const double* __restrict__ partials, unsigned int G, double* out, BaroFuse baro,
               int* err) {
    pdl_wait();
    pdl_trigger();
    __shared__ double res[kOut];
    __shared__ float2 red[kOut * 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (baro.on && threadIdx.x == 32) {
        const int s = *baro.counter;
        prefetch_l1(baro.field);
        prefetch_l1(baro.bs);
        prefetch_l1(reinterpret_cast<const char*>(baro.bs) + 128);
        prefetch_l1(&baro.fun->c);
        if (s >= 0 && s < baro.a.n_steps) prefetch_l1(baro.randoms + (int64_t)s * baro.a.stride);
    }
    const float2* part = reinterpret_cast<const float2*>(partials);
    DF acc[kOut];
#pragma unroll
    for (int k = 0; k < kOut; ++k) acc[k] = DF{0.0f, 0.0f};
    for (unsigned int b0 = threadIdx.x; b0 < G; b0 += kFinishRounds * kFinishThreads) {
        float2 x[kFinishRounds][kOut];
#pragma unroll
        for (int u = 0; u < kFinishRounds; ++u) {
            const unsigned int b = b0 + u * kFinishThreads;
#pragma unroll
            for (int k = 0; k < kOut; ++k)
                x[u][k] = b < G ? __ldcg(part + (size_t)k * G + b) : make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int u = 0; u < kFinishRounds; ++u)
#pragma unroll
            for (int k = 0; k < kOut; ++k) acc[k] = df_add(acc[k], DF{x[u][k].x, x[u][k].y});
    }
    warp_df_reduce<kOut>(acc);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < kOut; ++k) red[k * 32 + warp] = make_float2(acc[k].hi, acc[k].lo);
    }
    __syncthreads();
    if (warp == 0) {
        DF t[kOut];
#pragma unroll
        for (int k = 0; k < kOut; ++k) {
            const float2 x = lane < kFinishThreads / 32 ? red[k * 32 + lane] : make_float2(0.0f, 0.0f);
            t[k] = DF{x.x, x.y};
        }
        warp_df_reduce<kOut>(t);
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < kOut; ++k) res[k] = (double)t[k].hi + (double)t[k].lo;
        }
    }
    __syncthreads();
    if (threadIdx.x < kOut) out[threadIdx.x] = res[threadIdx.x];
    if (threadIdx.x == 0 && baro.on)
        scr_update(baro.a, res[9], baro.field, res, baro.randoms, baro.counter, baro.bs, baro.fun,
                   baro.state, err);
}

// ------------------------------------------------------------- planner ---
struct DSU {
    std::vector<int> p;
    explicit DSU(int64_t n) : p(n) { std::iota(p.begin(), p.end(), 0); }
    int find(int x) {
        while (p[x] != x) {
            p[x] = p[p[x]];
            x = p[x];
        }
        return x;
    }
    void join(int a, int b) {
        a = find(a);
        b = find(b);
        if (a != b) p[std::max(a, b)] = std::min(a, b);
    }
};

template <typename T>
int upload(T** dst, const std::vector<T>& src) {
    size_t n = src.size() ? src.size() : 1;
    if (cudaMalloc(dst, sizeof(T) * n) != cudaSuccess) return HPF_ERR_CUDA;
    if (!src.empty() &&
        cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return HPF_ERR_CUDA;
    return HPF_OK;
}

int grid_size(const hpf_respa_plan* p) {
    const int g = p->warp_mode ? (p->n_groups + kWarps - 1) / kWarps : p->n_groups;
    return g + p->n_free_blocks;
}

}  // namespace

extern "C" {

int hpf_respa_plan_permute(hpf_respa_plan* p, const int32_t* inv, int64_t n,
                           const int32_t* free_ids, int64_t n_free, int* d_err, void* stream) {
    if (!p || !inv || n != p->n_beads || (free_ids && n_free != p->n_free)) return HPF_ERR_ARG;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (p->n_bonded > 0) {
        const int blocks = (int)std::min<int64_t>((p->n_bonded + 255) / 256, 4 * 152);
        k_remap_ids<<<blocks, 256, 0, st>>>(p->bead_ids, p->n_bonded, inv, n, d_err);
        if (cudaGetLastError() != cudaSuccess) return HPF_ERR_CUDA;
    }
    if (p->n_free > 0) {
        if (free_ids) {
            if (cudaMemcpyAsync(p->free_ids, free_ids, sizeof(int32_t) * (size_t)p->n_free,
                                cudaMemcpyDeviceToDevice, st) != cudaSuccess)
                return HPF_ERR_CUDA;
        } else {
            const int blocks = (int)std::min<int64_t>((p->n_free + 255) / 256, 4 * 152);
            k_remap_ids<<<blocks, 256, 0, st>>>(p->free_ids, p->n_free, inv, n, d_err);
            if (cudaGetLastError() != cudaSuccess) return HPF_ERR_CUDA;
        }
    }
    return HPF_OK;
}

int hpf_respa_plan_counts(const hpf_respa_plan* p, int64_t* n_bonded, int64_t* n_free) {
    if (!p) return HPF_ERR_ARG;
    if (n_bonded) *n_bonded = p->n_bonded;
    if (n_free) *n_free = p->n_free;
    return HPF_OK;
}

int hpf_respa_plan_destroy(hpf_respa_plan* p) {
    if (!p) return HPF_OK;
    void* ptrs[] = {p->grp_bead, p->bead_ids, p->bead_inc, p->inc_list, p->grp_bond,
                    p->bond_ij,  p->bond_p,   p->grp_ang,  p->ang_ijk,  p->ang_p,
                    p->grp_dih,  p->dih_ijkl, p->dih_coeff, p->dih_trig, p->dih_tl,
                    p->dih_gid,
                    p->free_ids, p->partials};
    for (void* q : ptrs) cudaFree(q);
    if (p->free_stream) cudaStreamDestroy(p->free_stream);
    if (p->free_fork) cudaEventDestroy(p->free_fork);
    if (p->free_join) cudaEventDestroy(p->free_join);
    delete p;
    return HPF_OK;
}

int hpf_respa_plan_create(hpf_respa_plan** out, int64_t n, int64_t nb, const int32_t* ba,
                          const int32_t* bb, const float* br0, const float* bk, int64_t na,
                          const int32_t* aa, const int32_t* ab, const int32_t* ac,
                          const float* at0, const float* ak, int64_t nd, const int32_t* da,
                          const int32_t* db, const int32_t* dc, const int32_t* dd,
                          const float* dcoeff, const int32_t* dtype, const int32_t* dlast,
                          int max_group_beads) {
    if (!out || n < 0 || n > (int64_t)0x7fffffff || nb < 0 || na < 0 || nd < 0 ||
        max_group_beads < 1)
        return HPF_ERR_ARG;
    *out = nullptr;
    auto bad = [n](int32_t i) { return i < 0 || (int64_t)i >= n; };
    DSU dsu(n);
    std::vector<char> bonded(n, 0);
    for (int64_t t = 0; t < nb; ++t) {
        if (bad(ba[t]) || bad(bb[t])) return HPF_ERR_INDEX;
        dsu.join(ba[t], bb[t]);
        bonded[ba[t]] = bonded[bb[t]] = 1;
    }
    for (int64_t t = 0; t < na; ++t) {
        if (bad(aa[t]) || bad(ab[t]) || bad(ac[t])) return HPF_ERR_INDEX;
        dsu.join(aa[t], ab[t]);
        dsu.join(ab[t], ac[t]);
        bonded[aa[t]] = bonded[ab[t]] = bonded[ac[t]] = 1;
    }
    for (int64_t t = 0; t < nd; ++t) {
        if (bad(da[t]) || bad(db[t]) || bad(dc[t]) || bad(dd[t])) return HPF_ERR_INDEX;
        dsu.join(da[t], db[t]);
        dsu.join(db[t], dc[t]);
        dsu.join(dc[t], dd[t]);
        bonded[da[t]] = bonded[db[t]] = bonded[dc[t]] = bonded[dd[t]] = 1;
    }
    // components in order of their smallest bead (the DSU root is the minimum)
    std::vector<int> comp_size(n, 0);
    std::vector<int> free_ids;
    int largest = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (bonded[i]) comp_size[dsu.find((int)i)]++;
        else free_ids.push_back((int)i);
    }
    for (int64_t i = 0; i < n; ++i) largest = std::max(largest, comp_size[i]);
    // local bead indices are 16-bit; a CTA group must fit in shared memory
    if (largest > 32767) return HPF_ERR_NOT_IMPLEMENTED;
    const int cap = std::max(max_group_beads, largest);
    const int warp_mode = cap <= kWarpMaxBeads ? 1 : 0;
    std::vector<int> comp_grp(n, -1);
    std::vector<int> grp_beads;
    int cur = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (!bonded[i] || dsu.find((int)i) != (int)i) continue;
        const int sz = comp_size[i];
        if (grp_beads.empty() || cur + sz > cap) {
            grp_beads.push_back(0);
            cur = 0;
        }
        comp_grp[i] = (int)grp_beads.size() - 1;
        grp_beads.back() += sz;
        cur += sz;
    }
    const int G = (int)grp_beads.size();
    std::vector<int> grp_bead(G + 1, 0);
    for (int g = 0; g < G; ++g) grp_bead[g + 1] = grp_bead[g] + grp_beads[g];
    std::vector<int> bead_ids(grp_bead[G]);
    std::vector<int> local(n, -1), fill(grp_bead.begin(), grp_bead.end() - 1);
    for (int64_t i = 0; i < n; ++i) {
        if (!bonded[i]) continue;
        const int g = comp_grp[dsu.find((int)i)];
        local[i] = fill[g] - grp_bead[g];
        bead_ids[fill[g]++] = (int)i;
    }
    auto grp_of = [&](int i) { return comp_grp[dsu.find(i)]; };
    auto bucket = [&](int64_t cnt, auto first_bead, std::vector<int>& start,
                      std::vector<int64_t>& order) {
        std::vector<int> count(G + 1, 0);
        for (int64_t t = 0; t < cnt; ++t) count[grp_of(first_bead(t)) + 1]++;
        start.assign(G + 1, 0);
        for (int g = 0; g < G; ++g) start[g + 1] = start[g] + count[g + 1];
        std::vector<int> pos(start.begin(), start.end() - 1);
        order.assign(cnt, 0);
        for (int64_t t = 0; t < cnt; ++t) order[pos[grp_of(first_bead(t))]++] = t;
    };
    std::vector<int> sb, sa, sd;
    std::vector<int64_t> ob, oa, od;
    bucket(nb, [&](int64_t t) { return ba[t]; }, sb, ob);
    bucket(na, [&](int64_t t) { return aa[t]; }, sa, oa);
    bucket(nd, [&](int64_t t) { return da[t]; }, sd, od);
    std::vector<int> bond_ij(nb);
    std::vector<float2> bond_p(nb);
    for (int64_t k = 0; k < nb; ++k) {
        const int64_t t = ob[k];
        bond_ij[k] = local[ba[t]] | (local[bb[t]] << 16);
        bond_p[k] = make_float2(br0[t], bk[t]);
    }
    std::vector<int2> ang_ijk(na);
    std::vector<float2> ang_p(na);
    for (int64_t k = 0; k < na; ++k) {
        const int64_t t = oa[k];
        ang_ijk[k] = make_int2(local[aa[t]] | (local[ab[t]] << 16), local[ac[t]]);
        ang_p[k] = make_float2(at0[t], ak[t]);
    }
    std::vector<short4> dih_ijkl(nd);
    std::vector<float> dih_coeff(30 * nd);
    std::vector<int2> dih_tl(nd);
    std::vector<int> dih_gid(nd);
    for (int64_t k = 0; k < nd; ++k) {
        const int64_t t = od[k];
        dih_ijkl[k] = make_short4((short)local[da[t]], (short)local[db[t]], (short)local[dc[t]],
                                  (short)local[dd[t]]);
        for (int q = 0; q < 30; ++q) dih_coeff[30 * k + q] = dcoeff[30 * t + q];
        dih_tl[k] = make_int2(dtype[t], dlast[t]);
        dih_gid[k] = (int)t;
    }
    // incidence lists: per bead the (slot, sign) entries of the terms that
    // touch it; slots per group: bonds, then the angles' first and second
    // gradients, then the dihedrals' four corners, each corner-major (slot j
    // of term k at j * count + k), so that a warp's 32 terms write 32
    // consecutive slots; the entries per bead keep the terms' order
    std::vector<std::vector<int>> inc(grp_bead[G]);
    int mx_slots = 0, mx_bonds = 0, mx_angles = 0, mx_beads = 0, mx_inc = 0;
    for (int g = 0; g < G; ++g) {
        const int base = grp_bead[g];
        const int nbd_g = sb[g + 1] - sb[g], na_g = sa[g + 1] - sa[g], nd_g = sd[g + 1] - sd[g];
        for (int k = 0; k < nbd_g; ++k) {
            const int ij = bond_ij[sb[g] + k];
            inc[base + (ij & 0xffff)].push_back((k << 1) | 1);
            inc[base + (ij >> 16)].push_back(k << 1);
        }
        for (int k = 0; k < na_g; ++k) {
            const int2 q = ang_ijk[sa[g] + k];
            const int s0 = nbd_g + k, s1 = nbd_g + na_g + k;
            inc[base + (q.x & 0xffff)].push_back((s0 << 1) | 1);
            inc[base + (q.x >> 16)].push_back(s0 << 1);
            inc[base + (q.x >> 16)].push_back(s1 << 1);
            inc[base + q.y].push_back((s1 << 1) | 1);
        }
        for (int k = 0; k < nd_g; ++k) {
            const short4 q = dih_ijkl[sd[g] + k];
            const int s0 = nbd_g + 2 * na_g + k;
            const int li[4] = {q.x, q.y, q.z, q.w};
            for (int j = 0; j < 4; ++j) inc[base + li[j]].push_back((s0 + j * nd_g) << 1);
        }
        int ng = 0;
        for (int i = grp_bead[g]; i < grp_bead[g + 1]; ++i) ng += (int)inc[i].size();
        mx_inc = std::max(mx_inc, ng);
        mx_slots = std::max(mx_slots, nbd_g + 2 * na_g + 4 * nd_g);
        mx_bonds = std::max(mx_bonds, nbd_g);
        mx_angles = std::max(mx_angles, na_g);
        mx_beads = std::max(mx_beads, grp_beads[g]);
    }
    std::vector<int> bead_inc(grp_bead[G] + 1, 0), inc_list;
    for (int i = 0; i < grp_bead[G]; ++i) {
        bead_inc[i + 1] = bead_inc[i] + (int)inc[i].size();
        inc_list.insert(inc_list.end(), inc[i].begin(), inc[i].end());
    }
    hpf_respa_plan* p = new hpf_respa_plan();
    memset(p, 0, sizeof(*p));
    p->n_beads = n;
    p->n_groups = G;
    p->n_bonded = grp_bead[G];
    p->n_free = (int)free_ids.size();
    p->warp_mode = warp_mode;
    p->has_dih = nd > 0;
    p->mx_beads = std::max(mx_beads, 1);
    p->mx_slots = std::max(mx_slots, 1);
    p->mx_inc = std::max(mx_inc, 1);
    p->mx_bonds = std::max(mx_bonds, 1);
    p->mx_angles = std::max(mx_angles, 1);
    p->smem_group = group_smem_bytes(p->mx_beads, p->mx_slots, p->mx_inc, p->mx_bonds,
                                     p->mx_angles);
    p->smem = p->smem_group * (warp_mode ? kWarps : 1);
    if (p->smem > 227 * 1024) {
        delete p;
        return HPF_ERR_NOT_IMPLEMENTED;
    }
    const int grp_blocks = warp_mode ? (G + kWarps - 1) / kWarps : G;
    // free beads: a few per thread, over at least the SMs' worth of blocks
    // that the molecule groups leave (grid-stride loop inside)
    int nfb = (p->n_free + kThreads - 1) / kThreads;
    nfb = std::min(nfb, std::max(2 * 152, 152 * 8 - grp_blocks));
    if (p->n_free == 0) nfb = 0;
    p->n_free_blocks = nfb;
    int st = HPF_OK;
    if ((st = upload(&p->grp_bead, grp_bead)) || (st = upload(&p->bead_ids, bead_ids)) ||
        (st = upload(&p->bead_inc, bead_inc)) || (st = upload(&p->inc_list, inc_list)) ||
        (st = upload(&p->grp_bond, sb)) || (st = upload(&p->bond_ij, bond_ij)) ||
        (st = upload(&p->bond_p, bond_p)) || (st = upload(&p->grp_ang, sa)) ||
        (st = upload(&p->ang_ijk, ang_ijk)) || (st = upload(&p->ang_p, ang_p)) ||
        (st = upload(&p->grp_dih, sd)) || (st = upload(&p->dih_ijkl, dih_ijkl)) ||
        (st = upload(&p->dih_coeff, dih_coeff)) || (st = upload(&p->dih_tl, dih_tl)) ||
        (st = upload(&p->dih_gid, dih_gid)) || (st = upload(&p->free_ids, free_ids))) {
        hpf_respa_plan_destroy(p);
        return st;
    }
    if (cudaMalloc(&p->dih_trig, sizeof(float) * 30 * (size_t)std::max<int64_t>(nd, 1)) !=
        cudaSuccess) {
        hpf_respa_plan_destroy(p);
        return HPF_ERR_CUDA;
    }
    if (nd > 0) {
        k_dih_trig<<<(int)((nd + 127) / 128), 128>>>(p->dih_coeff, p->dih_trig, nd);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
            hpf_respa_plan_destroy(p);
            return HPF_ERR_CUDA;
        }
    }
    const int grid = grid_size(p);
    if (cudaMalloc(&p->partials, sizeof(double) * kOut * (size_t)std::max(grid, 1)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p->free_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->free_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->free_join, cudaEventDisableTiming) != cudaSuccess) {
        hpf_respa_plan_destroy(p);
        return HPF_ERR_CUDA;
    }
    if (p->smem > 48 * 1024) {
        // both variants (with and without the fused paint) of this plan's kernel
        const void* fns[2] = {
            warp_mode ? (p->has_dih ? (const void*)k_respa_warp<true, false>
                                    : (const void*)k_respa_warp<false, false>)
                      : (p->has_dih ? (const void*)k_respa_cta<true, false>
                                    : (const void*)k_respa_cta<false, false>),
            warp_mode ? (p->has_dih ? (const void*)k_respa_warp<true, true>
                                    : (const void*)k_respa_warp<false, true>)
                      : (p->has_dih ? (const void*)k_respa_cta<true, true>
                                    : (const void*)k_respa_cta<false, true>)};
        for (const void* fn : fns) {
            if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)p->smem) != cudaSuccess) {
                hpf_respa_plan_destroy(p);
                return HPF_ERR_CUDA;
            }
        }
    }
    *out = p;
    return HPF_OK;
}

int hpf_respa_plan_info(const hpf_respa_plan* p, int* n_groups, int* n_free,
                        int* max_group_beads) {
    if (!p) return HPF_ERR_ARG;
    if (n_groups) *n_groups = p->n_groups;
    if (n_free) *n_free = p->n_free;
    if (max_group_beads) *max_group_beads = p->mx_beads;
    return HPF_OK;
}

}  // extern "C"

namespace {

int respa_run(hpf_respa_plan* p, float* r, float* v, float* f_bonded,
              const float* const* slow_forces, int n_slow, double mass, double dt,
              int respa_inner, const double* box, float* dipoles, float* transfer, double* out,
              hpf_ctx* baro_ctx, const HpfScrArgs* baro, const double* field_sums,
              const double* randoms, int* counter, double* state, int* d_err, void* stream,
              const PaintFuse* pf) {
    if (!p || !r || !v || !f_bonded || !box || n_slow < 0 || n_slow > kMaxSlow ||
        (n_slow > 0 && !slow_forces) || !(mass > 0) || respa_inner < 1 ||
        (dipoles != nullptr) != (transfer != nullptr))
        return HPF_ERR_ARG;
    BaroFuse bf;
    memset(&bf, 0, sizeof(bf));
    if (baro) {
        if (!baro_ctx || !field_sums || !randoms || !counter || !state || !out ||
            baro->n_types != baro_ctx->T)
            return HPF_ERR_ARG;
        bf.on = 1;
        bf.a = *baro;
        bf.field = field_sums;
        bf.randoms = randoms;
        bf.counter = counter;
        bf.bs = baro_ctx->d_box;
        bf.fun = baro_ctx->d_fun;
        bf.state = state;
    }
    SlowForces sf;
    sf.n = n_slow;
    for (int q = 0; q < n_slow; ++q) {
        if (!slow_forces[q]) return HPF_ERR_ARG;
        sf.f[q] = slow_forces[q];
    }
    const int grid = grid_size(p);
    if (grid == 0) return HPF_OK;
    cudaStream_t st = as_stream(stream);
    const float h_out = (float)(0.5 * respa_inner * dt), hdt = (float)(0.5 * dt);
    PaintFuse pfv;
    memset(&pfv, 0, sizeof(pfv));
    if (pf) pfv = *pf;
    // with the paint fused in, the free beads run as a kernel of their own on
    // the plan's second stream, beside the group kernel, which is launched
    // first so that its blocks are placed before the free ones
    const bool split = pf && p->n_free_blocks > 0;
    const int ggrid = split ? grid - p->n_free_blocks : grid;
    const unsigned int G = (unsigned int)grid;
    if (split) HPF_CUDA_TRY(cudaEventRecord(p->free_fork, st));
    int rc = HPF_OK;
    if (ggrid > 0) {
#define HPF_RESPA(K)                                                                          \
    K<<<ggrid, kThreads, p->smem, st>>>(*p, r, v, f_bonded, sf, (float)mass, h_out, hdt,       \
                                        (float)dt, respa_inner, box, dipoles, transfer, out, 0, \
                                        pfv, G)
        if (p->warp_mode) {
            if (pf) {
                if (p->has_dih) HPF_RESPA((k_respa_warp<true, true>));
                else HPF_RESPA((k_respa_warp<false, true>));
            } else {
                if (p->has_dih) HPF_RESPA((k_respa_warp<true, false>));
                else HPF_RESPA((k_respa_warp<false, false>));
            }
        } else {
            if (pf) {
                if (p->has_dih) HPF_RESPA((k_respa_cta<true, true>));
                else HPF_RESPA((k_respa_cta<false, true>));
            } else {
                if (p->has_dih) HPF_RESPA((k_respa_cta<true, false>));
                else HPF_RESPA((k_respa_cta<false, false>));
            }
        }
#undef HPF_RESPA
        if (cudaGetLastError() != cudaSuccess) rc = HPF_ERR_CUDA;
    }
    if (split) {
        // the join is recorded whatever happens, so that a stream capture is
        // never left forked
        cudaError_t e = cudaStreamWaitEvent(p->free_stream, p->free_fork, 0);
        if (e == cudaSuccess) {
            k_respa_free<true><<<p->n_free_blocks, kThreads, 0, p->free_stream>>>(
                *p, r, v, sf, (float)mass, h_out, (float)dt, respa_inner, box, out, pfv, G,
                (unsigned int)ggrid);
            e = cudaGetLastError();
        }
        HPF_CUDA_TRY(cudaEventRecord(p->free_join, p->free_stream));
        if (e != cudaSuccess) rc = HPF_ERR_CUDA;
    }
    if (split) HPF_CUDA_TRY(cudaStreamWaitEvent(st, p->free_join, 0));
    if (rc != HPF_OK) return rc;
    if (out && launch_pdl(k_respa_finish, 1, kFinishThreads, 0, st,
                          static_cast<const double*>(p->partials), G, out, bf, d_err) !=
                   cudaSuccess)
        return HPF_ERR_CUDA;
    return HPF_OK;
}

}  // namespace

extern "C" {

int hpf_respa_step(hpf_respa_plan* p, float* r, float* v, float* f_bonded,
                   const float* const* slow_forces, int n_slow, double mass, double dt,
                   int respa_inner, const double* box, float* dipoles, float* transfer,
                   double* out, hpf_ctx* baro_ctx, const HpfScrArgs* baro,
                   const double* field_sums, const double* randoms, int* counter, double* state,
                   int* d_err, void* stream) {
    return respa_run(p, r, v, f_bonded, slow_forces, n_slow, mass, dt, respa_inner, box, dipoles,
                     transfer, out, baro_ctx, baro, field_sums, randoms, counter, state, d_err,
                     stream, nullptr);
}

int hpf_respa_step_paint(hpf_respa_plan* p, float* r, float* v, float* f_bonded,
                         const float* const* slow_forces, int n_slow, double mass, double dt,
                         int respa_inner, const double* box, float* dipoles, float* transfer,
                         double* out, hpf_ctx* field_ctx, const int32_t* types,
                         const float* charges, const HpfScrArgs* baro, const double* field_sums,
                         const double* randoms, int* counter, double* state, int* d_err,
                         void* stream) {
    // a semi-isotropic barostat moves the box under unscaled positions: its
    // grid coordinates change after the deposits, so it is refused
    if (baro && baro->mode != 0) return HPF_ERR_ARG;
    if (!field_ctx || !types || (p && field_ctx->M <= 0)) return HPF_ERR_ARG;
    PaintFuse pf;
    pf.acc = field_ctx->d_acc;
    pf.bs = field_ctx->d_box;
    pf.types = types;
    pf.charges = charges;
    pf.M = field_ctx->M;
    pf.T = field_ctx->T;
    pf.err = d_err ? d_err : field_ctx->d_err;
    return respa_run(p, r, v, f_bonded, slow_forces, n_slow, mass, dt, respa_inner, box, dipoles,
                     transfer, out, baro ? field_ctx : nullptr, baro, field_sums, randoms, counter,
                     state, d_err, stream, &pf);
}

int hpf_respa_forces(hpf_respa_plan* p, const float* r, float* f_bonded, const double* box,
                     double* out, int* d_err, void* stream) {
    if (!p || !r || !f_bonded || !box) return HPF_ERR_ARG;
    const int grid = p->warp_mode ? (p->n_groups + kWarps - 1) / kWarps : p->n_groups;
    if (grid == 0) return HPF_OK;
    cudaStream_t st = as_stream(stream);
    SlowForces sf;
    sf.n = 0;
    // v is neither read nor written in this mode; r is only read
    float* rr = const_cast<float*>(r);
    PaintFuse none;
    memset(&none, 0, sizeof(none));
#define HPF_RESPA_F(K)                                                                       \
    K<<<grid, kThreads, p->smem, st>>>(*p, rr, nullptr, f_bonded, sf, 1.0f, 0.0f, 0.0f, 0.0f, \
                                       1, box, nullptr, nullptr, out, 1, none,           \
                                       (unsigned int)grid)
    if (p->warp_mode) {
        if (p->has_dih) HPF_RESPA_F((k_respa_warp<true, false>));
        else HPF_RESPA_F((k_respa_warp<false, false>));
    } else {
        if (p->has_dih) HPF_RESPA_F((k_respa_cta<true, false>));
        else HPF_RESPA_F((k_respa_cta<false, false>));
    }
#undef HPF_RESPA_F
    HPF_LAUNCH_CHECK();
    if (out) {
        BaroFuse none;
        memset(&none, 0, sizeof(none));
        k_respa_finish<<<1, kFinishThreads, 0, st>>>(p->partials, (unsigned int)grid, out, none, d_err);
        HPF_LAUNCH_CHECK();
    }
    return HPF_OK;
}

}  // extern "C"

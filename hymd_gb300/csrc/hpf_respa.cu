// Fused rRESPA inner loop of HyMD on GB300 (hymd/main.py:802-887).
//
// Bonded terms never couple different molecules, so the whole inner loop --
// respa_inner x (half kick, drift, wrap, bonded forces, half kick) -- needs no
// grid-wide synchronisation if a group of threads owns whole molecules.  The
// planner (host C++) finds the molecules as connected components of the
// bonded terms, packs them into groups of at most `max_group_beads` beads and
// rewrites every term with group-local bead indices.  One launch then:
//   * molecule groups: load positions, velocities and bonded forces of the
//     group's beads into shared memory, apply the first outer half kick with
//     the slow forces, run all inner steps on chip, write back.  Groups of up
//     to 256 beads are run by one warp each (phases separated by __syncwarp);
//     larger ones by a whole CTA (__syncthreads);
//   * free beads (in no bonded term): per thread, the outer kick and
//     respa_inner drift/wrap steps (their bonded force is zero).
// Energies and virials of the last inner step (the ones the reference keeps,
// main.py:964-973) and sum v^2 are reduced in FP64 by the grid's last block,
// which can also run the isotropic SCR barostat (hymd/barostat_scr.py:34-132)
// right there, since the barostat follows the inner loop (main.py:889-963).
#include <algorithm>
#include <numeric>
#include <vector>

#include "hpf_internal.cuh"
#include "hpf_terms.cuh"

struct hpf_respa_plan {
    int64_t n_beads;
    int n_groups;        // molecule groups
    int n_free;
    int max_group_beads;
    int n_free_blocks;
    int warp_mode;       // 1: one warp per group, 0: one CTA per group
    int has_dih;
    size_t smem;         // dynamic shared memory per block
    // device arrays
    int* grp_bead;    // [n_groups+1]
    int* bead_ids;    // bonded beads, group-major
    int* grp_bond;    // [n_groups+1]
    short2* bond_ij;  // local indices
    float2* bond_p;   // (r0, k)
    int* grp_ang;
    short4* ang_ijk;
    float2* ang_p;    // (t0, k)
    int* grp_dih;
    short4* dih_ijkl;
    float* dih_coeff;  // 30 per term
    int2* dih_tl;      // (type, last)
    int* dih_gid;      // global dihedral index (dipole / transfer rows)
    int* free_ids;
    double* partials;
    unsigned int* ticket;
};

namespace {

constexpr int kThreads = 128;  // 4 warps
constexpr int kWarps = kThreads / 32;
constexpr int kMaxSlow = 4;
constexpr int kOut = 10;  // E_bond, pr_bond[3], E_angle, pr_angle[3], E_dihedral, sum v^2
constexpr int kWarpMaxBeads = 256;

struct SlowForces {
    const float* f[kMaxSlow];
    int n;
};

// Optional barostat run by the last block (all inner steps are done then).
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

// Group-local work shared by the warp and CTA variants.  `lane`/`width`
// enumerate the threads of the group; `sync()` separates the phases.
template <bool DIH, typename Sync>
__device__ __forceinline__ void run_group(const hpf_respa_plan& p, int grp, int lane, int width,
                                          float* rs, float* vs, float* fs, float* __restrict__ r,
                                          float* __restrict__ v, float* __restrict__ fb,
                                          const SlowForces& slow, float mass, float h_out,
                                          float hdt, float dt, int respa, const Box& bx,
                                          float* __restrict__ dipoles,
                                          float* __restrict__ transfer, float (&acc)[kOut],
                                          Sync sync) {
    const int s0 = p.grp_bead[grp], nb = p.grp_bead[grp + 1] - s0;
    const float inv_m = 1.0f / mass;
    for (int e = lane; e < 3 * nb; e += width) {
        const int i = e / 3, d = e - 3 * i;
        const int64_t g = 3 * (int64_t)p.bead_ids[s0 + i] + d;
        float x = v[g];
        for (int q = 0; q < slow.n; ++q) x = x + h_out * div_m(slow.f[q][g], mass, inv_m);
        vs[e] = x;
        rs[e] = r[g];
        fs[e] = fb[g];
    }
    sync();
    const int b0 = p.grp_bond[grp], b1 = p.grp_bond[grp + 1];
    const int a0 = p.grp_ang[grp], a1 = p.grp_ang[grp + 1];
    const int d0 = DIH ? p.grp_dih[grp] : 0, d1 = DIH ? p.grp_dih[grp + 1] : 0;
    for (int it = 0; it < respa; ++it) {
        const bool last_it = it == respa - 1;
        // closing half kick of the previous inner step (same forces), the
        // opening half kick of this one, drift and wrap; clear forces
        for (int i = lane; i < nb; i += width) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int e = 3 * i + d;
                const float a = div_m(fs[e], mass, inv_m);
                float x = vs[e];
                if (it > 0) x = x + hdt * a;
                x = x + hdt * a;
                vs[e] = x;
                rs[e] = wrapf(rs[e] + dt * x, bx.L[d]);
                fs[e] = 0.0f;
            }
        }
        sync();
        for (int t = b0 + lane; t < b1; t += width) {
            const short2 ij = p.bond_ij[t];
            const float2 pr = p.bond_p[t];
            float e;
            V3 vir;
            const V3 pa = v3(rs[3 * ij.x], rs[3 * ij.x + 1], rs[3 * ij.x + 2]);
            const V3 pb = v3(rs[3 * ij.y], rs[3 * ij.y + 1], rs[3 * ij.y + 2]);
            const V3 fa = bond_term(pa, pb, pr.x, pr.y, bx, e, vir);
            atomicAdd(fs + 3 * ij.x, -fa.x);
            atomicAdd(fs + 3 * ij.x + 1, -fa.y);
            atomicAdd(fs + 3 * ij.x + 2, -fa.z);
            atomicAdd(fs + 3 * ij.y, fa.x);
            atomicAdd(fs + 3 * ij.y + 1, fa.y);
            atomicAdd(fs + 3 * ij.y + 2, fa.z);
            if (last_it) {
                acc[0] += e;
                acc[1] += vir.x;
                acc[2] += vir.y;
                acc[3] += vir.z;
            }
        }
        for (int t = a0 + lane; t < a1; t += width) {
            const short4 q = p.ang_ijk[t];
            const float2 pr = p.ang_p[t];
            const V3 pa = v3(rs[3 * q.x], rs[3 * q.x + 1], rs[3 * q.x + 2]);
            const V3 pb = v3(rs[3 * q.y], rs[3 * q.y + 1], rs[3 * q.y + 2]);
            const V3 pc = v3(rs[3 * q.z], rs[3 * q.z + 1], rs[3 * q.z + 2]);
            V3 ga, gc, vir;
            float e;
            if (!angle_term(pa, pb, pc, pr.x, pr.y, bx, ga, gc, e, vir)) continue;
            atomicAdd(fs + 3 * q.x, -ga.x);
            atomicAdd(fs + 3 * q.x + 1, -ga.y);
            atomicAdd(fs + 3 * q.x + 2, -ga.z);
            atomicAdd(fs + 3 * q.z, -gc.x);
            atomicAdd(fs + 3 * q.z + 1, -gc.y);
            atomicAdd(fs + 3 * q.z + 2, -gc.z);
            atomicAdd(fs + 3 * q.y, ga.x + gc.x);
            atomicAdd(fs + 3 * q.y + 1, ga.y + gc.y);
            atomicAdd(fs + 3 * q.y + 2, ga.z + gc.z);
            if (last_it) {
                acc[4] += e;
                acc[5] += vir.x;
                acc[6] += vir.y;
                acc[7] += vir.z;
            }
        }
        if (DIH) {
            for (int t = d0 + lane; t < d1; t += width) {
                const short4 q = p.dih_ijkl[t];
                const int2 tl = p.dih_tl[t];
                const int li[4] = {q.x, q.y, q.z, q.w};
                V3 pos[4];
                for (int j = 0; j < 4; ++j)
                    pos[j] = v3(rs[3 * li[j]], rs[3 * li[j] + 1], rs[3 * li[j] + 2]);
                float* dip = nullptr;
                float* tmx = nullptr;
                if (last_it && dipoles) {
                    const int64_t gd = p.dih_gid[t];
                    dip = dipoles + 12 * gd;
                    tmx = transfer + 54 * gd;
                    for (int j = 0; j < 12; ++j) dip[j] = 0.0f;
                    for (int j = 0; j < 54; ++j) tmx[j] = 0.0f;
                }
                V3 F[4];
                float e;
                dihedral_term(pos[0], pos[1], pos[2], pos[3], p.dih_coeff + 30 * (int64_t)t, tl.x,
                              tl.y, (last_it && dipoles) ? 1 : 0, bx, F, e, dip, tmx);
                for (int j = 0; j < 4; ++j) {
                    atomicAdd(fs + 3 * li[j], F[j].x);
                    atomicAdd(fs + 3 * li[j] + 1, F[j].y);
                    atomicAdd(fs + 3 * li[j] + 2, F[j].z);
                }
                if (last_it) acc[8] += e;
            }
        }
        sync();
    }
    // closing half kick of the last inner step, write back
    for (int e = lane; e < 3 * nb; e += width) {
        const int i = e / 3, d = e - 3 * i;
        const int64_t g = 3 * (int64_t)p.bead_ids[s0 + i] + d;
        const float a = div_m(fs[e], mass, inv_m);
        const float x = vs[e] + hdt * a;
        v[g] = x;
        r[g] = rs[e];
        fb[g] = fs[e];
        acc[9] = fmaf(x, x, acc[9]);
    }
}

__device__ __forceinline__ void free_beads(const hpf_respa_plan& p, int fblock, float* __restrict__ r,
                                           float* __restrict__ v, const SlowForces& slow,
                                           float mass, float h_out, float dt, int respa,
                                           const Box& bx, float (&acc)[kOut]) {
    const int stride = p.n_free_blocks * kThreads;
    for (int j = fblock * kThreads + threadIdx.x; j < p.n_free; j += stride) {
        const int64_t g = 3 * (int64_t)p.free_ids[j];
        for (int d = 0; d < 3; ++d) {
            float x = v[g + d];
            for (int q = 0; q < slow.n; ++q)
                x = x + h_out * div_m(slow.f[q][g + d], mass, 1.0f / mass);
            float y = r[g + d];
            for (int it = 0; it < respa; ++it) y = wrapf(y + dt * x, bx.L[d]);
            v[g + d] = x;
            r[g + d] = y;
            acc[9] = fmaf(x, x, acc[9]);
        }
    }
}

__device__ __forceinline__ void scr_epilogue(const BaroFuse& f, const double* out, int* err) {
    scr_update(f.a, out[9], f.field, out, f.randoms, f.counter, f.bs, f.fun, f.state, err);
}

template <bool DIH>
__global__ void __launch_bounds__(kThreads)
k_respa_warp(hpf_respa_plan p, float* __restrict__ r, float* __restrict__ v,
             float* __restrict__ fb, SlowForces slow, float mass, float h_out, float hdt, float dt,
             int respa, const double* __restrict__ box, float* __restrict__ dipoles,
             float* __restrict__ transfer, double* out, BaroFuse baro, int* err) {
    extern __shared__ float smem[];
    const Box bx = load_box(box);
    float acc[kOut];
#pragma unroll
    for (int k = 0; k < kOut; ++k) acc[k] = 0.0f;
    const int n_grp_blocks = (p.n_groups + kWarps - 1) / kWarps;
    if ((int)blockIdx.x < n_grp_blocks) {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const int grp = blockIdx.x * kWarps + warp;
        if (grp < p.n_groups) {
            float* base = smem + (size_t)warp * 9 * p.max_group_beads;
            run_group<DIH>(p, grp, lane, 32, base, base + 3 * p.max_group_beads,
                           base + 6 * p.max_group_beads, r, v, fb, slow, mass, h_out, hdt, dt,
                           respa, bx, dipoles, transfer, acc, WarpSync());
        }
    } else {
        free_beads(p, blockIdx.x - n_grp_blocks, r, v, slow, mass, h_out, dt, respa, bx, acc);
    }
    if (!out) return;
    if (grid_reduce_store_f<kOut>(acc, p.partials, p.ticket, out) && baro.on)
        scr_epilogue(baro, out, err);
}

template <bool DIH>
__global__ void __launch_bounds__(kThreads)
k_respa_cta(hpf_respa_plan p, float* __restrict__ r, float* __restrict__ v,
            float* __restrict__ fb, SlowForces slow, float mass, float h_out, float hdt, float dt,
            int respa, const double* __restrict__ box, float* __restrict__ dipoles,
            float* __restrict__ transfer, double* out, BaroFuse baro, int* err) {
    extern __shared__ float smem[];
    const Box bx = load_box(box);
    float acc[kOut];
#pragma unroll
    for (int k = 0; k < kOut; ++k) acc[k] = 0.0f;
    if ((int)blockIdx.x < p.n_groups) {
        const int nb = p.max_group_beads;
        run_group<DIH>(p, blockIdx.x, threadIdx.x, kThreads, smem, smem + 3 * nb, smem + 6 * nb,
                       r, v, fb, slow, mass, h_out, hdt, dt, respa, bx, dipoles, transfer, acc,
                       CtaSync());
    } else {
        free_beads(p, blockIdx.x - p.n_groups, r, v, slow, mass, h_out, dt, respa, bx, acc);
    }
    if (!out) return;
    if (grid_reduce_store_f<kOut>(acc, p.partials, p.ticket, out) && baro.on)
        scr_epilogue(baro, out, err);
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

int hpf_respa_plan_destroy(hpf_respa_plan* p) {
    if (!p) return HPF_OK;
    void* ptrs[] = {p->grp_bead, p->bead_ids, p->grp_bond, p->bond_ij, p->bond_p, p->grp_ang,
                    p->ang_ijk, p->ang_p, p->grp_dih, p->dih_ijkl, p->dih_coeff, p->dih_tl,
                    p->dih_gid, p->free_ids, p->partials, p->ticket};
    for (void* q : ptrs) cudaFree(q);
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
    // a group must fit in shared memory (36 bytes per bead); a warp takes
    // groups of up to kWarpMaxBeads beads, a CTA up to ~6400
    const int hard = (227 * 1024) / 36;
    if (largest > hard) return HPF_ERR_NOT_IMPLEMENTED;
    int cap = std::max(max_group_beads, largest);
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
    std::vector<short2> bond_ij(nb);
    std::vector<float2> bond_p(nb);
    for (int64_t k = 0; k < nb; ++k) {
        const int64_t t = ob[k];
        bond_ij[k] = make_short2((short)local[ba[t]], (short)local[bb[t]]);
        bond_p[k] = make_float2(br0[t], bk[t]);
    }
    std::vector<short4> ang_ijk(na);
    std::vector<float2> ang_p(na);
    for (int64_t k = 0; k < na; ++k) {
        const int64_t t = oa[k];
        ang_ijk[k] = make_short4((short)local[aa[t]], (short)local[ab[t]], (short)local[ac[t]], 0);
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
    hpf_respa_plan* p = new hpf_respa_plan();
    memset(p, 0, sizeof(*p));
    p->n_beads = n;
    p->n_groups = G;
    p->n_free = (int)free_ids.size();
    p->warp_mode = warp_mode;
    p->has_dih = nd > 0;
    int mx = 0;
    for (int g = 0; g < G; ++g) mx = std::max(mx, grp_beads[g]);
    p->max_group_beads = std::max(mx, 1);
    p->smem = sizeof(float) * 9 * (size_t)p->max_group_beads * (warp_mode ? kWarps : 1);
    const int grp_blocks = warp_mode ? (G + kWarps - 1) / kWarps : G;
    int nfb = (p->n_free + kThreads - 1) / kThreads;
    nfb = std::min(nfb, std::max(1, 152 * 8 - grp_blocks));
    if (p->n_free == 0) nfb = 0;
    p->n_free_blocks = nfb;
    int st = HPF_OK;
    if ((st = upload(&p->grp_bead, grp_bead)) || (st = upload(&p->bead_ids, bead_ids)) ||
        (st = upload(&p->grp_bond, sb)) || (st = upload(&p->bond_ij, bond_ij)) ||
        (st = upload(&p->bond_p, bond_p)) || (st = upload(&p->grp_ang, sa)) ||
        (st = upload(&p->ang_ijk, ang_ijk)) || (st = upload(&p->ang_p, ang_p)) ||
        (st = upload(&p->grp_dih, sd)) || (st = upload(&p->dih_ijkl, dih_ijkl)) ||
        (st = upload(&p->dih_coeff, dih_coeff)) || (st = upload(&p->dih_tl, dih_tl)) ||
        (st = upload(&p->dih_gid, dih_gid)) || (st = upload(&p->free_ids, free_ids))) {
        hpf_respa_plan_destroy(p);
        return st;
    }
    const int grid = grid_size(p);
    if (cudaMalloc(&p->partials, sizeof(double) * kOut * (size_t)std::max(grid, 1)) != cudaSuccess ||
        cudaMalloc(&p->ticket, sizeof(unsigned int)) != cudaSuccess ||
        cudaMemset(p->ticket, 0, sizeof(unsigned int)) != cudaSuccess) {
        hpf_respa_plan_destroy(p);
        return HPF_ERR_CUDA;
    }
    if (p->smem > 48 * 1024) {
        const void* fn = warp_mode ? (p->has_dih ? (const void*)k_respa_warp<true>
                                                 : (const void*)k_respa_warp<false>)
                                   : (p->has_dih ? (const void*)k_respa_cta<true>
                                                 : (const void*)k_respa_cta<false>);
        if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem) !=
            cudaSuccess) {
            hpf_respa_plan_destroy(p);
            return HPF_ERR_CUDA;
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
    if (max_group_beads) *max_group_beads = p->max_group_beads;
    return HPF_OK;
}

int hpf_respa_step(hpf_respa_plan* p, float* r, float* v, float* f_bonded,
                   const float* const* slow_forces, int n_slow, double mass, double dt,
                   int respa_inner, const double* box, float* dipoles, float* transfer,
                   double* out, hpf_ctx* baro_ctx, const HpfScrArgs* baro,
                   const double* field_sums, const double* randoms, int* counter, double* state,
                   int* d_err, void* stream) {
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
#define HPF_RESPA(K)                                                                          \
    K<<<grid, kThreads, p->smem, st>>>(*p, r, v, f_bonded, sf, (float)mass, h_out, hdt,        \
                                       (float)dt, respa_inner, box, dipoles, transfer, out, bf, \
                                       d_err)
    if (p->warp_mode) {
        if (p->has_dih) HPF_RESPA(k_respa_warp<true>);
        else HPF_RESPA(k_respa_warp<false>);
    } else {
        if (p->has_dih) HPF_RESPA(k_respa_cta<true>);
        else HPF_RESPA(k_respa_cta<false>);
    }
#undef HPF_RESPA
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

}  // extern "C"

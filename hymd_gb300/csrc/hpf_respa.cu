// Fused rRESPA inner loop of HyMD on GB300 (hymd/main.py:802-887).
//
// Bonded terms never couple different molecules, so the whole inner loop --
// respa_inner x (half kick, drift, wrap, bonded forces, half kick) -- needs no
// grid-wide synchronisation if each CTA owns whole molecules.  The planner
// (host C++) finds the molecules as connected components of the bonded
// terms, packs them into blocks of at most `max_block_beads` beads, and
// rewrites every term with block-local bead indices.  One launch then:
//   * molecule blocks: load positions, velocities and bonded forces of the
//     block's beads into shared memory, apply the first outer half kick with
//     the slow forces, run all inner steps on chip (shared-memory force
//     accumulation, __syncthreads between phases), write back;
//   * free beads (in no bonded term): per thread, the outer kick and
//     respa_inner drift/wrap steps (their bonded force is zero).
// Energies and virials of the last inner step (the ones the reference keeps,
// main.py:964-973) are reduced in FP64 deterministically.
#include <algorithm>
#include <numeric>
#include <vector>

#include "hpf_internal.cuh"
#include "hpf_terms.cuh"

struct hpf_respa_plan {
    int64_t n_beads;
    int n_mol_blocks;
    int n_free;
    int max_block_beads;
    int n_free_blocks;
    size_t smem;
    // device arrays
    int* blk_bead;    // [n_mol_blocks+1]
    int* bead_ids;    // bonded beads, block-major
    int* blk_bond;    // [n_mol_blocks+1]
    short2* bond_ij;  // local indices
    float2* bond_p;   // (r0, k)
    int* blk_ang;
    short4* ang_ijk;
    float2* ang_p;    // (t0, k)
    int* blk_dih;
    short4* dih_ijkl;
    float* dih_coeff;  // 30 per term
    int2* dih_tl;      // (type, last)
    int* dih_gid;      // global dihedral index (dipole / transfer rows)
    int* free_ids;
    double* partials;
    unsigned int* ticket;
};

namespace {

// 128 threads per block: molecule blocks are small (a few hundred beads), so
// several of them share an SM and their __syncthreads-separated phases
// overlap.
constexpr int kThreads = 128;
constexpr int kMaxSlow = 4;
constexpr int kOut = 9;  // E_bond, pr_bond[3], E_angle, pr_angle[3], E_dihedral

struct SlowForces {
    const float* f[kMaxSlow];
    int n;
};

__device__ __forceinline__ float wrapf(float x, float L) {
    float m = fmodf(x, L);
    if (m < 0.0f) m += L;
    return m;
}

__global__ void __launch_bounds__(kThreads)
k_respa(hpf_respa_plan p, float* __restrict__ r, float* __restrict__ v, float* __restrict__ fb,
        SlowForces slow, float mass, float h_out, float hdt, float dt, int respa,
        const double* __restrict__ box, float* __restrict__ dipoles, float* __restrict__ transfer,
        double* out, int* err) {
    extern __shared__ float smem[];
    const Box bx = load_box(box);
    float acc[kOut];  // a thread adds a few terms; FP64 from the warp sums up
#pragma unroll
    for (int k = 0; k < kOut; ++k) acc[k] = 0.0f;
    const int tid = threadIdx.x;
    if ((int)blockIdx.x < p.n_mol_blocks) {
        const int b = blockIdx.x;
        const int s0 = p.blk_bead[b], nb = p.blk_bead[b + 1] - s0;
        float* rs = smem;            // [3*nb]
        float* vs = smem + 3 * nb;   // [3*nb]
        float* fs = smem + 6 * nb;   // [3*nb]
        for (int e = tid; e < 3 * nb; e += kThreads) {
            const int i = e / 3, d = e - 3 * i;
            const int64_t g = 3 * (int64_t)p.bead_ids[s0 + i] + d;
            float x = v[g];
            for (int q = 0; q < slow.n; ++q) x = x + h_out * (slow.f[q][g] / mass);
            vs[e] = x;
            rs[e] = r[g];
            fs[e] = fb[g];
        }
        __syncthreads();
        const int b0 = p.blk_bond[b], b1 = p.blk_bond[b + 1];
        const int a0 = p.blk_ang[b], a1 = p.blk_ang[b + 1];
        const int d0 = p.blk_dih[b], d1 = p.blk_dih[b + 1];
        for (int it = 0; it < respa; ++it) {
            const bool last_it = it == respa - 1;
            // closing half kick of the previous inner step (same forces), the
            // opening half kick of this one, drift and wrap; clear forces
            for (int e = tid; e < 3 * nb; e += kThreads) {
                const float a = fs[e] / mass;
                float x = vs[e];
                if (it > 0) x = x + hdt * a;
                x = x + hdt * a;
                vs[e] = x;
                rs[e] = wrapf(rs[e] + dt * x, bx.L[e % 3]);
                fs[e] = 0.0f;
            }
            __syncthreads();
            for (int t = b0 + tid; t < b1; t += kThreads) {
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
            for (int t = a0 + tid; t < a1; t += kThreads) {
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
            for (int t = d0 + tid; t < d1; t += kThreads) {
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
            __syncthreads();
        }
        // closing half kick of the last inner step, write back
        for (int e = tid; e < 3 * nb; e += kThreads) {
            const int i = e / 3, d = e - 3 * i;
            const int64_t g = 3 * (int64_t)p.bead_ids[s0 + i] + d;
            const float a = fs[e] / mass;
            v[g] = vs[e] + hdt * a;
            r[g] = rs[e];
            fb[g] = fs[e];
        }
    } else {
        // free beads: zero bonded force, so each inner step is a pure drift
        const int fb0 = ((int)blockIdx.x - p.n_mol_blocks) * kThreads;
        const int stride = p.n_free_blocks * kThreads;
        for (int j = fb0 + tid; j < p.n_free; j += stride) {
            const int64_t g = 3 * (int64_t)p.free_ids[j];
            for (int d = 0; d < 3; ++d) {
                float x = v[g + d];
                for (int q = 0; q < slow.n; ++q) x = x + h_out * (slow.f[q][g + d] / mass);
                float y = r[g + d];
                for (int it = 0; it < respa; ++it) y = wrapf(y + dt * x, bx.L[d]);
                v[g + d] = x;
                r[g + d] = y;
            }
        }
    }
    if (out) grid_reduce_store_f<kOut>(acc, p.partials, p.ticket, out);
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

}  // namespace

extern "C" {

int hpf_respa_plan_destroy(hpf_respa_plan* p) {
    if (!p) return HPF_OK;
    void* ptrs[] = {p->blk_bead, p->bead_ids, p->blk_bond, p->bond_ij, p->bond_p, p->blk_ang,
                    p->ang_ijk, p->ang_p, p->blk_dih, p->dih_ijkl, p->dih_coeff, p->dih_tl,
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
                          int max_block_beads) {
    if (!out || n < 0 || n > (int64_t)0x7fffffff || nb < 0 || na < 0 || nd < 0 ||
        max_block_beads < 1)
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
    for (int64_t i = 0; i < n; ++i) {
        if (bonded[i]) comp_size[dsu.find((int)i)]++;
        else free_ids.push_back((int)i);
    }
    // hard limit: the block must fit in shared memory (36 bytes per bead)
    const int hard = (227 * 1024) / 36;
    std::vector<int> comp_block(n, -1);
    std::vector<int> block_beads;  // bead count per block
    int cur = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (!bonded[i] || dsu.find((int)i) != (int)i) continue;
        const int sz = comp_size[i];
        if (sz > hard) return HPF_ERR_NOT_IMPLEMENTED;
        if (block_beads.empty() || cur + sz > max_block_beads) {
            block_beads.push_back(0);
            cur = 0;
        }
        comp_block[i] = (int)block_beads.size() - 1;
        block_beads.back() += sz;
        cur += sz;
    }
    const int B = (int)block_beads.size();
    std::vector<int> blk_bead(B + 1, 0);
    for (int b = 0; b < B; ++b) blk_bead[b + 1] = blk_bead[b] + block_beads[b];
    std::vector<int> bead_ids(blk_bead[B]);
    std::vector<int> local(n, -1), fill(blk_bead.begin(), blk_bead.end() - 1);
    for (int64_t i = 0; i < n; ++i) {
        if (!bonded[i]) continue;
        const int b = comp_block[dsu.find((int)i)];
        local[i] = fill[b] - blk_bead[b];
        bead_ids[fill[b]++] = (int)i;
    }
    auto blk_of = [&](int i) { return comp_block[dsu.find(i)]; };
    auto bucket = [&](int64_t cnt, auto first_bead, std::vector<int>& start,
                      std::vector<int64_t>& order) {
        std::vector<int> count(B + 1, 0);
        for (int64_t t = 0; t < cnt; ++t) count[blk_of(first_bead(t)) + 1]++;
        start.assign(B + 1, 0);
        for (int b = 0; b < B; ++b) start[b + 1] = start[b] + count[b + 1];
        std::vector<int> pos(start.begin(), start.end() - 1);
        order.assign(cnt, 0);
        for (int64_t t = 0; t < cnt; ++t) order[pos[blk_of(first_bead(t))]++] = t;
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
    p->n_mol_blocks = B;
    p->n_free = (int)free_ids.size();
    int mx = 0;
    for (int b = 0; b < B; ++b) mx = std::max(mx, block_beads[b]);
    p->max_block_beads = mx;
    p->smem = sizeof(float) * 9 * (size_t)std::max(mx, 1);
    int nfb = (p->n_free + kThreads - 1) / kThreads;
    nfb = std::min(nfb, std::max(1, 152 * 8 - B));
    if (p->n_free == 0) nfb = 0;
    p->n_free_blocks = nfb;
    int st = HPF_OK;
    if ((st = upload(&p->blk_bead, blk_bead)) || (st = upload(&p->bead_ids, bead_ids)) ||
        (st = upload(&p->blk_bond, sb)) || (st = upload(&p->bond_ij, bond_ij)) ||
        (st = upload(&p->bond_p, bond_p)) || (st = upload(&p->blk_ang, sa)) ||
        (st = upload(&p->ang_ijk, ang_ijk)) || (st = upload(&p->ang_p, ang_p)) ||
        (st = upload(&p->blk_dih, sd)) || (st = upload(&p->dih_ijkl, dih_ijkl)) ||
        (st = upload(&p->dih_coeff, dih_coeff)) || (st = upload(&p->dih_tl, dih_tl)) ||
        (st = upload(&p->dih_gid, dih_gid)) || (st = upload(&p->free_ids, free_ids))) {
        hpf_respa_plan_destroy(p);
        return st;
    }
    const int grid = B + nfb;
    if (cudaMalloc(&p->partials, sizeof(double) * kOut * (size_t)std::max(grid, 1)) != cudaSuccess ||
        cudaMalloc(&p->ticket, sizeof(unsigned int)) != cudaSuccess ||
        cudaMemset(p->ticket, 0, sizeof(unsigned int)) != cudaSuccess) {
        hpf_respa_plan_destroy(p);
        return HPF_ERR_CUDA;
    }
    if (p->smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_respa, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)p->smem) != cudaSuccess) {
        hpf_respa_plan_destroy(p);
        return HPF_ERR_CUDA;
    }
    *out = p;
    return HPF_OK;
}

int hpf_respa_plan_info(const hpf_respa_plan* p, int* n_mol_blocks, int* n_free,
                        int* max_block_beads) {
    if (!p) return HPF_ERR_ARG;
    if (n_mol_blocks) *n_mol_blocks = p->n_mol_blocks;
    if (n_free) *n_free = p->n_free;
    if (max_block_beads) *max_block_beads = p->max_block_beads;
    return HPF_OK;
}

int hpf_respa_step(hpf_respa_plan* p, float* r, float* v, float* f_bonded,
                   const float* const* slow_forces, int n_slow, double mass, double dt,
                   int respa_inner, const double* box, float* dipoles, float* transfer,
                   double* out, int* d_err, void* stream) {
    if (!p || !r || !v || !f_bonded || !box || n_slow < 0 || n_slow > kMaxSlow ||
        (n_slow > 0 && !slow_forces) || !(mass > 0) || respa_inner < 1 ||
        (dipoles != nullptr) != (transfer != nullptr))
        return HPF_ERR_ARG;
    SlowForces sf;
    sf.n = n_slow;
    for (int q = 0; q < n_slow; ++q) {
        if (!slow_forces[q]) return HPF_ERR_ARG;
        sf.f[q] = slow_forces[q];
    }
    const int grid = p->n_mol_blocks + p->n_free_blocks;
    if (grid == 0) return HPF_OK;
    k_respa<<<grid, kThreads, p->smem, as_stream(stream)>>>(
        *p, r, v, f_bonded, sf, (float)mass, (float)(0.5 * respa_inner * dt), (float)(0.5 * dt),
        (float)dt, respa_inner, box, dipoles, transfer, out, d_err);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

}  // extern "C"

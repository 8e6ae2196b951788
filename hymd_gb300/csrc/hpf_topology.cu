// Bonded-term discovery of HyMD's prepare_bonds_old (hymd/force.py:325-505)
// on the device.
//
// The reference builds one networkx graph per molecule (rescanning every
// particle for each molecule) and walks it: all_pairs_shortest_path gives the
// bonds (paths of 2 nodes) and angles (paths of 3), find_all_paths
// (force.py:267-277) the 4-node paths matched against the dihedral types.
// The order of the resulting lists is fixed by those traversals, and the
// packed arrays of prepare_bonds keep it.  Here one thread walks one molecule
// and reproduces the same traversals, so the terms come out in the same
// order:
//   * nodes in insertion order: each member (ascending local index) and then
//     the partners in its bond row, as networkx's add_node / add_edge insert
//     them; neighbour lists in edge insertion order;
//   * per start node (in node order) a breadth-first search to depth 2 with
//     neighbours in insertion order (networkx's single-source shortest path):
//     depth-1 nodes j with gid(j) > gid(i) give bonds, depth-2 nodes angles
//     through the node they were discovered from; every matching type, in
//     the configuration's order, adds one term;
//   * the depth-first 4-node simple paths from the start node, each matched
//     forward against the dihedral types.  The reference skips a path whose
//     reversed term is already listed (same coefficients and type); that
//     term exists exactly when the path's last node comes earlier in node
//     order and the reversed names match a type of the same class.
// bb_index (force.py:501-502): the last type-1 dihedral of each molecule.
//
// Two launches: the first counts each molecule's terms, the host turns the
// counts into offsets, the second writes the terms there.  Names and term
// types arrive as small integers; the host maps names and parameters.
#include <algorithm>

#include "hpf_internal.cuh"

namespace {

constexpr int kTopoThreads = 128;

struct TopoArgs {
    int n_mol;
    int64_t n_beads;
    const int* mol_start;   // [n_mol + 1] slot ranges
    const int* slot_bead;   // slot -> local bead
    const int* bead_slot;   // local bead -> slot
    const long long* gid;   // local bead -> global index (node key)
    const int* name_id;     // local bead -> name id
    const int* partners;    // [n_beads][max_partners] local beads, -1 = none
    int max_partners;
    const int* bond_types;  // [nbt][2] name ids (-1: name absent)
    int nbt;
    const int* angle_types;  // [nat][3]
    int nat;
    const int* dih_types;  // [ndt][4]
    const int* dih_class;  // [ndt] equal for equal (coefficients, type)
    const int* dih_bb;     // [ndt] 1 for dihedral type 1
    int ndt;
    int* scratch;
    int* counts;        // [n_mol][3]
    const int* offsets;  // [n_mol][3] (write pass)
    int* bonds;          // [B][3]: i, j, type
    int* angles;         // [A][4]: i, mid, j, type
    int* dihedrals;      // [D][5]: a, b, c, d, type
    int* bb;             // [n_mol]: global index of the last type-1 dihedral, or -1
    int* err;
};

template <bool WRITE>
__global__ void __launch_bounds__(kTopoThreads) k_topology(TopoArgs a) {
    const int64_t N = a.n_beads;
    int* rank = a.scratch;
    int* order = a.scratch + N;
    int* deg = a.scratch + 2 * N;
    int* visit = a.scratch + 3 * N;
    int* parent = a.scratch + 4 * N;
    int* queue = a.scratch + 5 * N;
    int* adj = a.scratch + 6 * N;  // [N][HPF_TOPO_MAX_DEGREE]
    constexpr int D = HPF_TOPO_MAX_DEGREE;
    const int stride = gridDim.x * blockDim.x;
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < a.n_mol; m += stride) {
        const int s0 = a.mol_start[m], s1 = a.mol_start[m + 1];
        for (int s = s0; s < s1; ++s) {
            rank[s] = -1;
            deg[s] = 0;
            visit[s] = -1;
        }
        int R = 0;
        bool ok = true;
        auto add_node = [&](int s) {
            if (rank[s] < 0) {
                rank[s] = R;
                order[s0 + R] = s;
                ++R;
            }
        };
        auto add_adj = [&](int u, int v) {
            for (int q = 0; q < deg[u]; ++q)
                if (adj[(int64_t)u * D + q] == v) return true;
            if (deg[u] == D) return false;
            adj[(int64_t)u * D + deg[u]] = v;
            deg[u] += 1;
            return true;
        };
        for (int s = s0; s < s1 && ok; ++s) {
            const int b = a.slot_bead[s];
            add_node(s);
            for (int q = 0; q < a.max_partners; ++q) {
                const int p = a.partners[(int64_t)b * a.max_partners + q];
                if (p < 0) continue;
                const int t = p < N ? a.bead_slot[p] : -1;
                if (t < s0 || t >= s1) {  // partner outside this molecule
                    hpf_flag(a.err, HPF_ERR_INDEX);
                    ok = false;
                    break;
                }
                if (t == s) continue;  // a self-bond adds no path
                add_node(t);
                if (!add_adj(s, t) || !add_adj(t, s)) {
                    hpf_flag(a.err, HPF_ERR_NOT_IMPLEMENTED);
                    ok = false;
                    break;
                }
            }
        }
        int nb = 0, na = 0, nd = 0, last_bb = -1;
        const int ob = WRITE ? a.offsets[3 * m] : 0, oa = WRITE ? a.offsets[3 * m + 1] : 0,
                  od = WRITE ? a.offsets[3 * m + 2] : 0;
        for (int r = 0; ok && r < R; ++r) {
            const int i = order[s0 + r];
            const int bi = a.slot_bead[i];
            const long long gi = a.gid[bi];
            const int ni = a.name_id[bi];
            // breadth-first search to depth 2, discovery order in queue
            visit[i] = r;
            int n1 = 0;
            for (int q = 0; q < deg[i]; ++q) {
                const int w = adj[(int64_t)i * D + q];
                if (visit[w] != r) {
                    visit[w] = r;
                    parent[w] = i;
                    queue[s0 + n1++] = w;
                }
            }
            int n2 = n1;
            for (int e = 0; e < n1; ++e) {
                const int v = queue[s0 + e];
                for (int q = 0; q < deg[v]; ++q) {
                    const int w = adj[(int64_t)v * D + q];
                    if (visit[w] != r) {
                        visit[w] = r;
                        parent[w] = v;
                        queue[s0 + n2++] = w;
                    }
                }
            }
            for (int e = 0; e < n1; ++e) {
                const int bj = a.slot_bead[queue[s0 + e]];
                if (!(a.gid[bj] > gi)) continue;
                const int nj = a.name_id[bj];
                for (int k = 0; k < a.nbt; ++k) {
                    const int t1 = a.bond_types[2 * k], t2 = a.bond_types[2 * k + 1];
                    if ((ni == t1 && nj == t2) || (ni == t2 && nj == t1)) {
                        if (WRITE) {
                            int* o = a.bonds + 3 * (int64_t)(ob + nb);
                            o[0] = bi;
                            o[1] = bj;
                            o[2] = k;
                        }
                        ++nb;
                    }
                }
            }
            for (int e = n1; e < n2; ++e) {
                const int j = queue[s0 + e];
                const int bj = a.slot_bead[j];
                if (!(a.gid[bj] > gi)) continue;
                const int bm = a.slot_bead[parent[j]];
                const int nj = a.name_id[bj], nm = a.name_id[bm];
                for (int k = 0; k < a.nat; ++k) {
                    const int* t = a.angle_types + 3 * k;
                    if (nm == t[1] && ((ni == t[0] && nj == t[2]) || (ni == t[2] && nj == t[0]))) {
                        if (WRITE) {
                            int* o = a.angles + 4 * (int64_t)(oa + na);
                            o[0] = bi;
                            o[1] = bm;
                            o[2] = bj;
                            o[3] = k;
                        }
                        ++na;
                    }
                }
            }
            if (a.ndt == 0) continue;
            // 4-node simple paths i-w1-w2-w3, depth first
            for (int q1 = 0; q1 < deg[i]; ++q1) {
                const int w1 = adj[(int64_t)i * D + q1];
                const int n1n = a.name_id[a.slot_bead[w1]];
                for (int q2 = 0; q2 < deg[w1]; ++q2) {
                    const int w2 = adj[(int64_t)w1 * D + q2];
                    if (w2 == i) continue;
                    const int n2n = a.name_id[a.slot_bead[w2]];
                    for (int q3 = 0; q3 < deg[w2]; ++q3) {
                        const int w3 = adj[(int64_t)w2 * D + q3];
                        if (w3 == w1 || w3 == i) continue;
                        const int n3n = a.name_id[a.slot_bead[w3]];
                        for (int k = 0; k < a.ndt; ++k) {
                            const int* t = a.dih_types + 4 * k;
                            if (!(ni == t[0] && n1n == t[1] && n2n == t[2] && n3n == t[3]))
                                continue;
                            bool listed = false;
                            if (rank[w3] < r) {
                                for (int k2 = 0; k2 < a.ndt && !listed; ++k2) {
                                    const int* u = a.dih_types + 4 * k2;
                                    listed = a.dih_class[k2] == a.dih_class[k] && n3n == u[0] &&
                                             n2n == u[1] && n1n == u[2] && ni == u[3];
                                }
                            }
                            if (listed) continue;
                            if (WRITE) {
                                int* o = a.dihedrals + 5 * (int64_t)(od + nd);
                                o[0] = bi;
                                o[1] = a.slot_bead[w1];
                                o[2] = a.slot_bead[w2];
                                o[3] = a.slot_bead[w3];
                                o[4] = k;
                            }
                            if (a.dih_bb[k]) last_bb = od + nd;
                            ++nd;
                        }
                    }
                }
            }
        }
        if (WRITE) {
            a.bb[m] = last_bb;
        } else {
            a.counts[3 * m] = nb;
            a.counts[3 * m + 1] = na;
            a.counts[3 * m + 2] = nd;
        }
    }
}

}  // namespace

extern "C" {

int64_t hpf_topology_scratch_ints(int64_t n_beads) {
    return n_beads < 0 ? -1 : (6 + HPF_TOPO_MAX_DEGREE) * n_beads;
}

int hpf_topology_terms(int64_t n_beads, int n_mol, const int* mol_start, const int* slot_bead,
                       const int* bead_slot, const long long* gid, const int* name_id,
                       const int* partners, int max_partners, const int* bond_types, int n_bond_types,
                       const int* angle_types, int n_angle_types, const int* dih_types,
                       const int* dih_class, const int* dih_bb, int n_dih_types, int* scratch,
                       int* counts, const int* offsets, int* bonds, int* angles, int* dihedrals,
                       int* bb, int* d_err, void* stream) {
    if (n_beads < 0 || n_beads > 0x7fffffff || n_mol < 0 || max_partners < 0 ||
        n_bond_types < 0 || n_angle_types < 0 || n_dih_types < 0)
        return HPF_ERR_ARG;
    if (n_mol == 0) return HPF_OK;
    if (!mol_start || !slot_bead || !bead_slot || !gid || !name_id || !scratch || !d_err ||
        (max_partners > 0 && !partners) || (n_bond_types > 0 && !bond_types) ||
        (n_angle_types > 0 && !angle_types) ||
        (n_dih_types > 0 && (!dih_types || !dih_class || !dih_bb)))
        return HPF_ERR_ARG;
    if (offsets ? (!bonds || !angles || !dihedrals || !bb) : !counts) return HPF_ERR_ARG;
    TopoArgs a;
    a.n_mol = n_mol;
    a.n_beads = n_beads;
    a.mol_start = mol_start;
    a.slot_bead = slot_bead;
    a.bead_slot = bead_slot;
    a.gid = gid;
    a.name_id = name_id;
    a.partners = partners;
    a.max_partners = max_partners;
    a.bond_types = bond_types;
    a.nbt = n_bond_types;
    a.angle_types = angle_types;
    a.nat = n_angle_types;
    a.dih_types = dih_types;
    a.dih_class = dih_class;
    a.dih_bb = dih_bb;
    a.ndt = n_dih_types;
    a.scratch = scratch;
    a.counts = counts;
    a.offsets = offsets;
    a.bonds = bonds;
    a.angles = angles;
    a.dihedrals = dihedrals;
    a.bb = bb;
    a.err = d_err;
    const int grid = (int)std::min<int64_t>((n_mol + kTopoThreads - 1) / kTopoThreads, 152 * 16);
    cudaStream_t st = as_stream(stream);
    if (offsets) k_topology<true><<<grid, kTopoThreads, 0, st>>>(a);
    else k_topology<false><<<grid, kTopoThreads, 0, st>>>(a);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

}  // extern "C"

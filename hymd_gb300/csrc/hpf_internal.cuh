// Internal device helpers shared by the hpf_gb300 translation units.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include "../../include/hpf_gb300.h"

#define HPF_MAX_TYPES 16

// Box state kept in device memory so that graphs replayed after a device-side
// barostat rescale see the new box.  The first five doubles are part of the
// C ABI (hpf_ctx_box_state): L[3], V, dV.
struct BoxState {
    double L[3];
    double V;
    double dV;
    float Lf[3];      // float box, used by the position wrap
    float ih_hi[3];   // n_d / L_d split into two floats (hi + lo)
    float ih_lo[3];
    float kf[3];      // 2 pi / L_d
    float inv_dV;
    int n[3];
    int pad;
    double inv_M;     // 1 / (n0 n1 n2)
};

// Quadratic functional w = 1/2 phi.Q.phi + b.phi + c (per context).
struct Functional {
    float Q[HPF_MAX_TYPES * HPF_MAX_TYPES];
    float b[HPF_MAX_TYPES];
    double Qd[HPF_MAX_TYPES * HPF_MAX_TYPES];
    double bd[HPF_MAX_TYPES];
    double c;
    double sigma2_half_d;  // 0.5 * sigma^2
    float sigma2_half;
    float pad;
};

struct hpf_ctx {
    int n0, n1, n2, T;
    int64_t M, Mc;
    int device;
    BoxState* d_box;          // device
    BoxState h_box;           // host mirror (last value set from the host)
    Functional* d_fun;        // device
    Functional h_fun;
    unsigned long long* d_acc;  // paint accumulators int64[T+1][M] (the +1 is for charges)
    float* d_grid;            // real scratch float[3T][M] (densities / force mesh)
    float2* d_spec;           // spectral scratch float2[3T][Mc]
    float2* d_spec_phi;       // raw density spectra float2[T][Mc]
    double* d_ws;             // reduction workspace (HPF_OUT_DOUBLES)
    int* d_err;               // first device error code
    void* fft_work;
    size_t fft_work_size;
    // FP64 energy path (created on first use, outside graph capture)
    cufftHandle plan_d2z;     // batch T+1: T densities + charges
    bool has_d2z;
    double* d_grid64;         // double[T+1][M]
    double2* d_spec64;        // double2[T+1][Mc]
    cufftHandle plan_r2c[HPF_MAX_TYPES + 1];   // batch b at index b (created lazily)
    cufftHandle plan_c2r[3 * HPF_MAX_TYPES + 2];
    bool has_r2c[HPF_MAX_TYPES + 1];
    bool has_c2r[3 * HPF_MAX_TYPES + 2];
    // PIC_Spectral_GPE scratch (created on first use): grids rho~ / q, total
    // density, eta[3], X, E[3], psi (10 M floats); spectra (4 Mc); a
    // reduction workspace and a pinned host word for the convergence test
    float* gpe_grid;
    float2* gpe_spec;
    double* gpe_ws;
    double* gpe_host;
    // the polarisation iteration as a CUDA graph: a while node whose body
    // (r2c, field map, 3 c2r, update, convergence test) sets its own
    // condition on the device; built on first use on gpe_cap, rebuilt when
    // the iterated grid, mixing, tolerance, measure or iteration cap change
    cudaGraph_t gpe_graph;
    cudaGraphExec_t gpe_exec;
    cudaStream_t gpe_cap;
    const float* gpe_key_pol;
    double gpe_key_mix, gpe_key_crit;
    int gpe_key_kind, gpe_key_max;
    // fused spectral passes: twiddle tables exp(-2 pi i m / 512) and
    // exp(-2 pi i m / 768), k-space tile width, partial sums + ticket
    float2* d_tw;
    double* d_spec_ws;
    int spec_W, spec_tiles, spec_max_tiles;
    int spec_W_pic, spec_tiles_pic;  // the charge k-space pass's own tile width
    int spec_ok;     // the mesh qualifies and the scratch exists
    int spec_fused;  // use them (default when spec_ok)
    // the charge chain's own scratch, so that it can run beside the density
    // chain (hpf_field_pic_step; created on first use, outside capture):
    // spectra float2[1 + 2][Mc], grids float[4][M] (psi, E_x, E_y, E_z),
    // partial sums + ticket; a second stream and the fork / join events
    float2* pic_spec_phi;
    float2* pic_spec;
    float* pic_grid;
    double* pic_spec_ws;
    cudaStream_t pic_stream;
    cudaEvent_t pic_fork, pic_join;
};

// Buffers of one chain of the fused spectral passes: spectra in (pass A ->
// B) and out (B -> C), the real force grids of pass C, and the partial sums
// + ticket of pass B's reduction.
struct SpecBufs {
    float2* spec_phi;
    float2* spec;
    float* grid;
    double* ws;
};

// Paint deposits are integers in units of 2^-24 of a particle's weight (a
// charge of up to 2^7 e keeps a deposit inside int32).
constexpr float kFixScale = 16777216.0f;          // 2^24
constexpr float kFixInv = 5.9604644775390625e-8f;  // 2^-24

// int64 -> float without the 64-bit conversion instruction (FP64 pipe on
// GB300): magnitude split into 32-bit halves, one FMA.  Deterministic.
__device__ __forceinline__ float fix_to_float(long long x) {
    const bool neg = x < 0;
    const unsigned long long a = neg ? (unsigned long long)(-x) : (unsigned long long)x;
    const float f = fmaf((float)(unsigned)(a >> 32), 4294967296.0f, (float)(unsigned)a);
    return neg ? -f : f;
}

// Fused spectral passes (hpf_spectral.cu): eligibility, setup at context
// creation, and accumulators -> force mesh (c->d_grid, [3T][M]).
bool spectral_eligible(const hpf_ctx* c);
int spectral_setup(hpf_ctx* c);
bool spectral_tile_ok(const hpf_ctx* c, int W);
int spectral_set_tile(hpf_ctx* c, int W);
int spectral_field_force(hpf_ctx* c, const float* type_scale, double* sums, cudaStream_t st);
// real_in non-NULL: the input is that real grid (float[M]) instead of the
// charge accumulator; filter = false drops H(k) from the Poisson map (the GPE
// solve's psi = scale (q + pol) / k^2).
int spectral_pic(hpf_ctx* c, const SpecBufs& b, float four_pi_fac, bool want_psi, double* sums,
                 cudaStream_t st, const float* real_in = nullptr, bool filter = true);
// words of a pass-B partial-sum buffer (partials of the narrowest tile + ticket)
size_t spectral_ws_words(const hpf_ctx* c);

#define HPF_REDUCE_GRID 304  // blocks of a reduction kernel (2 per SM on 152 SMs)

// Layout of a reduction workspace (see HPF_OUT_DOUBLES in the C ABI header).
__host__ __device__ inline double* ws_partials(double* ws) { return ws + 8; }
__host__ __device__ inline unsigned int* ws_ticket(double* ws) {
    return reinterpret_cast<unsigned int*>(ws + 8 + 8 * HPF_REDUCE_BLOCKS);
}

static inline int reduce_grid(int64_t work, int threads) {
    int64_t b = (work + threads - 1) / threads;
    if (b < 1) b = 1;
    // two blocks per SM are plenty for a grid-stride reduction, and keep the
    // last block's FP64 pass over the partials short
    if (b > HPF_REDUCE_GRID) b = HPF_REDUCE_GRID;
    return (int)b;
}

// Derived box quantities, shared by the host setter and the device barostat.
__host__ __device__ inline void fill_box_state(BoxState& s, double L0, double L1, double L2,
                                               const int n[3]) {
    const double Ls[3] = {L0, L1, L2};
    s.V = L0 * L1 * L2;
    s.dV = s.V / ((double)n[0] * (double)n[1] * (double)n[2]);
    for (int d = 0; d < 3; ++d) {
        s.L[d] = Ls[d];
        s.n[d] = n[d];
        s.Lf[d] = (float)Ls[d];
        double ih = (double)n[d] / Ls[d];
        s.ih_hi[d] = (float)ih;
        s.ih_lo[d] = (float)(ih - (double)s.ih_hi[d]);
        s.kf[d] = (float)(2.0 * 3.14159265358979323846 / Ls[d]);
    }
    s.inv_dV = (float)(1.0 / s.dV);
    s.inv_M = 1.0 / ((double)n[0] * (double)n[1] * (double)n[2]);
}

// Record the first device-side error code (out-of-range index, non-finite
// input, exhausted table); the host reads it with hpf_get_error.
__device__ __forceinline__ void hpf_flag(int* err, int code) {
    if (err) atomicCAS(err, 0, code);
}

// FP64 reciprocal from the FP32 one and two Newton steps (FMA only): FP64
// division is a long instruction sequence on GB300's thin FP64 pipe, and the
// single-thread epilogues below sit on the critical path of a step.
__device__ __forceinline__ double rcp_d(double x) {
    double r = (double)(1.0f / (float)x);
    r = r * fma(-x, r, 2.0);
    r = r * fma(-x, r, 2.0);
    return r;
}

// Device-side box update (barostat) from the new float box lengths: the same
// quantities as fill_box_state.  Run by one thread on the critical path of a
// step, so only V and dV are formed in FP64 (GB300's FP64 pipe is narrow);
// n/L is the double-float quotient hi + lo from FP32 operations (FMA
// residual), equal to the host's split to within an ulp of lo.
__device__ __forceinline__ void fill_box_state_dev(BoxState& s, float L0, float L1, float L2) {
    const float Ls[3] = {L0, L1, L2};
    s.V = (double)L0 * (double)L1 * (double)L2;
    s.dV = s.V * s.inv_M;
    for (int d = 0; d < 3; ++d) {
        const float L = Ls[d], nd = (float)s.n[d];
        s.L[d] = (double)L;
        s.Lf[d] = L;
        const float hi = nd / L;
        s.ih_hi[d] = hi;
        s.ih_lo[d] = fmaf(-hi, L, nd) / L;
        s.kf[d] = 6.28318530717958647692f / L;
    }
    s.inv_dV = ((float)s.n[0] * (float)s.n[1] * (float)s.n[2]) / (float)s.V;
}

// CSVR scale factors (hymd/thermostat.py:167-219, Bussi-Parrinello 2008 form)
// from the per-group sums ws[4g..4g+3] = (sum v_x, sum v_y, sum v_z, sum v^2)
// taken before the thermostat, run by one thread once the sums are final.
// The reference visits the coupling groups in order and each visit changes
// the velocities the next one sees:
//   * with centre-of-mass removal (and more than one particle in the group),
//     K is the group's kinetic energy about its current COM velocity c, and
//     only the group's particles move: v <- (v - c) alpha + c;
//   * otherwise K is the whole system's current kinetic energy and every
//     particle is scaled: v <- alpha v.
// Each visit is affine in the pre-thermostat velocities, so the composition
// is tracked per particle group h as v_final = A_h v + B_h, and the current
// sums of a later visit follow from the pre-thermostat ones.  state[4h] = A_h,
// state[4h+1..3] = B_h (what hpf_csvr_scale applies), state[8+g] += K (alpha^2 - 1)
// (config.thermostat_work).  Every particle belongs to exactly one group (the
// reference's check_thermostat_coupling_groups), so the group sums cover the
// whole system.  alpha^2 is formed in FP32, as the O(1) factor has no
// cancellation; K and the composed transforms are FP64.
__device__ __forceinline__ void csvr_update(const HpfCsvrArgs& a, const double* ws,
                                            const double* randoms, int* counter, double* state,
                                            int* err) {
    const int s = *counter;
    const bool ok = s >= 0 && s < a.n_steps;
    if (!ok) hpf_flag(err, HPF_ERR_INDEX);
    const bool act = !(a.every > 1 && (s + 1) % a.every != 0);
    const int ng = a.n_groups < 1 ? 1 : (a.n_groups > 2 ? 2 : a.n_groups);
    double A[2] = {1.0, 1.0};
    double B[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    for (int g = 0; act && g < ng; ++g) {
        const double N = a.count[g];
        const bool com = a.remove_com && N > 1.0;
        double cnow[3] = {0.0, 0.0, 0.0};
        double K;
        if (com) {
            const double iN = 1.0 / N;
            double c2 = 0.0;
            for (int d = 0; d < 3; ++d) {
                const double c0 = ws[4 * g + d] * iN;
                c2 += c0 * c0;
                cnow[d] = A[g] * c0 + B[g][d];
            }
            K = 0.5 * a.mass * A[g] * A[g] * (ws[4 * g + 3] - N * c2);
        } else {
            K = 0.0;
            for (int h = 0; h < ng; ++h) {
                double bs = 0.0, bb = 0.0;
                for (int d = 0; d < 3; ++d) {
                    bs += B[h][d] * ws[4 * h + d];
                    bb += B[h][d] * B[h][d];
                }
                K += A[h] * A[h] * ws[4 * h + 3] + 2.0 * A[h] * bs + a.count[h] * bb;
            }
            K *= 0.5 * a.mass;
        }
        const float Kt = (float)(1.5 * a.gas_constant * N * a.target_temperature);
        const float Nf = 3.0f * (float)N;
        const float R = ok ? (float)randoms[(int64_t)s * a.stride + a.offset + 2 * g] : 0.0f;
        const float S = ok ? (float)randoms[(int64_t)s * a.stride + a.offset + 2 * g + 1] : Nf - 1.0f;
        const float c = (float)a.c;
        const float q = Kt / (Nf * (float)K);
        const float alpha2 = c + (1.0f - c) * (S + R * R) * q + 2.0f * R * sqrtf(c * (1.0f - c) * q);
        const double al = (double)sqrtf(alpha2);
        if (com) {
            A[g] *= al;
            for (int d = 0; d < 3; ++d) B[g][d] = al * (B[g][d] - cnow[d]) + cnow[d];
        } else {
            for (int h = 0; h < ng; ++h) {
                A[h] *= al;
                for (int d = 0; d < 3; ++d) B[h][d] *= al;
            }
        }
        state[8 + g] += K * ((double)alpha2 - 1.0);
    }
    for (int h = 0; h < 2; ++h) {
        state[4 * h] = A[h];
        for (int d = 0; d < 3; ++d) state[4 * h + 1 + d] = B[h][d];
    }
    if (a.advance) *counter = s + 1;
}

// SCR barostat step run by one thread once all sums are final: isotropic
// (hymd/barostat_scr.py:34-132) or semi-isotropic with z normal (:133-284).
// The pressure components are added in FP64; with the k = 0 densities
// mean_t = m_t N_t / V the field part of p0 + p1 reduces to
//   -W/V + A + (Q mean + b).mean = A/2 + (1/2 mc.Q.mc) / V^2 - c.
// `bonded` holds {E_bond, bond_pr[3], E_angle, angle_pr[3]}.  The box is kept
// in float32 values, as the reference's float32 box_size array.
// state[12] = alpha (semi-isotropic: lateral alpha_L), state[13] = P
// (semi-isotropic: P_L), state[14] = alpha_N, state[15] = P_N,
// state[10] = surface tension L_z/2 (P_N - P_L) (bar nm).
__device__ __forceinline__ void scr_update(const HpfScrArgs& a, double sum_v2,
                                           const double* field, const double* bonded,
                                           const double* randoms, int* counter, BoxState* bs,
                                           const Functional* fun, double* state, int* err) {
    const int s = *counter;
    const bool ok = s >= 0 && s < a.n_steps;
    if (!ok) hpf_flag(err, HPF_ERR_INDEX);
    state[12] = 1.0;
    state[14] = 1.0;
    if (!(a.every > 1 && (s + 1) % a.every != 0)) {
        const double V = bs->V;
        const double iV = rcp_d(V);
        const double A = field[0];
        const double p_kin = (2.0 / 3.0) * iV * (0.5 * a.mass * sum_v2);
        const double p01 = 0.5 * A + a.half_mQm * iV * iV - fun->c;
        const double sig2 = 2.0 * fun->sigma2_half_d;
        double ptot[3];
        for (int d = 0; d < 3; ++d)
            ptot[d] = p_kin + p01 - sig2 * field[1 + d] + (bonded[1 + d] + bonded[5 + d]) * iV;
        const float itau = 1.0f / (float)a.tau_p;
        const float nb = (float)a.n_b, bdt = (float)a.beta * (float)a.dt_outer;
        const float kT = (float)a.gas_constant * (float)a.target_temperature;
        if (a.mode == 0) {
            // the reference averages p_tot[-3:-1], i.e. the x and y components
            const double P = 0.5 * (ptot[0] + ptot[1]) * 16.61;
            const float R = ok ? (float)randoms[(int64_t)s * a.stride] : 0.0f;
            const float noise = sqrtf(2.0f * nb * kT * bdt * nb * (float)iV * itau) * R;
            const float log_alpha = -(nb * bdt) * itau * (float)(a.target_pressure - P) + noise;
            const double alpha = (double)expf(log_alpha / 3.0f);
            fill_box_state_dev(*bs, (float)(bs->L[0] * alpha), (float)(bs->L[1] * alpha),
                               (float)(bs->L[2] * alpha));
            state[12] = alpha;
            state[13] = P;
        } else {
            const double PL = 0.5 * (ptot[0] + ptot[1]) * 16.61, PN = ptot[2] * 16.61;
            double L[3] = {bs->L[0], bs->L[1], bs->L[2]};
            const double gamma = 0.5 * L[2] * (PN - PL);
            const float Rxy = ok ? (float)randoms[(int64_t)s * a.stride] : 0.0f;
            const float Rz = ok ? (float)randoms[(int64_t)s * a.stride + 1] : 0.0f;
            double aL = 1.0, aN = 1.0;
            if (a.couple_l) {
                const float iVf = (float)rcp_d(L[0] * L[1] * L[2]);
                const float noise = sqrtf(4.0f * nb * kT * bdt * nb * iVf * itau / 3.0f) * Rxy;
                const float log_alpha =
                    -2.0f * nb * bdt * itau / 3.0f *
                        (float)(a.target_pressure - PL - gamma / L[2]) + noise;
                aL = (double)expf(log_alpha / 2.0f);
                L[0] = (double)(float)(L[0] * aL);
                L[1] = (double)(float)(L[1] * aL);
            }
            if (a.couple_n) {
                // the volume after the lateral rescale, as in the reference
                const float iVf = (float)rcp_d(L[0] * L[1] * L[2]);
                const float noise = sqrtf(2.0f * nb * kT * bdt * nb * iVf * itau / 3.0f) * Rz;
                const float log_alpha =
                    -nb * bdt * itau / 3.0f * (float)(a.target_pressure_n - PN) + noise;
                aN = (double)expf(log_alpha);
                L[2] = (double)(float)(L[2] * aN);
            }
            fill_box_state_dev(*bs, (float)L[0], (float)L[1], (float)L[2]);
            state[10] = gamma;
            state[12] = aL;
            state[13] = PL;
            state[14] = aN;
            state[15] = PN;
        }
    }
    if (a.advance) *counter = s + 1;
}

#define HPF_CUDA_TRY(x)                                   \
    do {                                                  \
        cudaError_t e_ = (x);                             \
        if (e_ != cudaSuccess) return HPF_ERR_CUDA;       \
    } while (0)

#define HPF_LAUNCH_CHECK()                                \
    do {                                                  \
        cudaError_t e_ = cudaGetLastError();              \
        if (e_ != cudaSuccess) return HPF_ERR_CUDA;       \
    } while (0)

static inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Programmatic dependent launch (sm_90 and later).  A kernel started with
// launch_pdl may be scheduled before its predecessor on the stream has
// finished: it calls pdl_wait() before anything else, which returns once the
// predecessor grid has completed and its memory operations are visible.  A
// kernel calls pdl_trigger() when its main work is done, so that its
// successor's blocks are scheduled while it drains (a block that exits
// without it counts as triggered).  Both are no-ops in a kernel launched the
// ordinary way.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}


// Grid coordinate s = x * n/L split into a node index and a fraction in
// [0,1), using only FP32 arithmetic.  n/L is held as hi+lo floats and the
// product's rounding error is recovered with an FMA, so the fraction is
// accurate to ~1e-7 absolute (a plain float product would lose up to
// n * 6e-8 near the far edge of the box).
__device__ __forceinline__ void grid_coord(float x, float ih_hi, float ih_lo, int n, int& i,
                                           float& frac) {
    float s = x * ih_hi;
    float e = fmaf(x, ih_hi, -s);          // exact residual of the product
    float fl = floorf(s);
    float f = (s - fl) + fmaf(x, ih_lo, e);
    if (f >= 1.0f) { f -= 1.0f; fl += 1.0f; }
    if (f < 0.0f) { f += 1.0f; fl -= 1.0f; }
    int ii = (int)fl;
    ii %= n;
    if (ii < 0) ii += n;
    i = ii;
    frac = f;
}

// Mesh geometry of a CIC deposit, loaded once per thread from a BoxState.
struct CicMesh {
    int n0, n1, n2;
    float h0, h1, h2, l0, l1, l2;  // n_d / L_d as hi + lo floats
};
__device__ __forceinline__ CicMesh cic_mesh(const BoxState* bs) {
    CicMesh m;
    m.n0 = bs->n[0];
    m.n1 = bs->n[1];
    m.n2 = bs->n[2];
    m.h0 = bs->ih_hi[0];
    m.h1 = bs->ih_hi[1];
    m.h2 = bs->ih_hi[2];
    m.l0 = bs->ih_lo[0];
    m.l1 = bs->ih_lo[1];
    m.l2 = bs->ih_lo[2];
    return m;
}

// CIC deposit of weight q at (x, y, z) into one grid of int64 accumulators
// ([n0][n1][n2], units of 2^-24 of a unit weight): the 8 corner weights
// converted with an FP32 -> int32 rounding (a 64-bit conversion runs on the
// FP64 pipe) and added with 64-bit atomics, zero deposits skipped.  Integer
// sums do not depend on the order of the deposits: the grid is
// bit-deterministic whichever kernel paints and in whatever order.
__device__ __forceinline__ void cic_deposit(const CicMesh& m, float x, float y, float z, float q,
                                            unsigned long long* __restrict__ base) {
    int ix, iy, iz;
    float fx, fy, fz;
    grid_coord(x, m.h0, m.l0, m.n0, ix, fx);
    grid_coord(y, m.h1, m.l1, m.n1, iy, fy);
    grid_coord(z, m.h2, m.l2, m.n2, iz, fz);
    const int jx = ix + 1 == m.n0 ? 0 : ix + 1;
    const int jy = iy + 1 == m.n1 ? 0 : iy + 1;
    const int jz = iz + 1 == m.n2 ? 0 : iz + 1;
    const float wx[2] = {1.0f - fx, fx}, wy[2] = {1.0f - fy, fy}, wz[2] = {1.0f - fz, fz};
    const int xs[2] = {ix, jx}, ys[2] = {iy, jy}, zs[2] = {iz, jz};
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const int64_t row = ((int64_t)xs[a] * m.n1 + ys[b]) * m.n2;
            const float wab = q * wx[a] * wy[b];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const long long v = (long long)__float2int_rn(wab * wz[c] * kFixScale);
                if (v != 0) atomicAdd(base + row + zs[c], (unsigned long long)v);
            }
        }
}

// A paint fused into another kernel (the rRESPA inner loop): each bead is
// deposited where that kernel leaves its final position -- its type's
// density grid and, with charges, the charge grid after the T density
// grids -- with the deposits of k_paint (cic_deposit), so the accumulators
// end up bit-identical to those of a separate paint.
struct PaintFuse {
    unsigned long long* acc;  // int64 accumulators [T + 1][M]
    const BoxState* bs;       // mesh of the field context
    const int32_t* types;     // bead types
    const float* charges;     // bead charges, or nullptr (no charge grid)
    int64_t M;
    int T;
    int* err;                 // first error code (non-finite position, type)
};

__device__ __forceinline__ void paint_bead(const PaintFuse& pf, const CicMesh& m, int64_t i,
                                           float x, float y, float z) {
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) {
        hpf_flag(pf.err, HPF_ERR_NONFINITE);
        return;
    }
    const int t = pf.types[i];
    if (t < 0 || t >= pf.T) {
        hpf_flag(pf.err, HPF_ERR_INDEX);
        return;
    }
    cic_deposit(m, x, y, z, 1.0f, pf.acc + (int64_t)t * pf.M);
    if (pf.charges) {
        const float q = pf.charges[i];
        if (q != 0.0f) cic_deposit(m, x, y, z, q, pf.acc + (int64_t)pf.T * pf.M);
    }
}

// Warp + block reduction of K doubles; thread 0 returns the block totals.
template <int K>
__device__ __forceinline__ void block_reduce(double (&v)[K], double* smem /* K*32 */) {
    // the K shuffle trees advance level by level together (latencies overlap)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        double t[K];
#pragma unroll
        for (int k = 0; k < K; ++k) t[k] = __shfl_down_sync(0xffffffffu, v[k], o);
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] += t[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) smem[k * 32 + warp] = v[k];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = lane < nw ? smem[k * 32 + lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double t[K];
#pragma unroll
            for (int k = 0; k < K; ++k) t[k] = __shfl_down_sync(0xffffffffu, v[k], o);
#pragma unroll
            for (int k = 0; k < K; ++k) v[k] += t[k];
        }
    }
}

// Compensated ("double-float") sum of two (hi, lo) FP32 pairs: TwoSum of the
// high parts, then the low parts folded in and renormalised.  About 48
// significant bits, using only the FP32 pipe.
struct DF {
    float hi, lo;
};

__device__ __forceinline__ DF df_add(DF a, DF b) {
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e += a.lo + b.lo;
    const float hi = s + e;
    return DF{hi, e - (hi - s)};
}

__device__ __forceinline__ DF df_shfl_down(DF v, int o) {
    return DF{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
}

// Warp sum of K double-float values (shuffle tree, lane 0 holds the sums).
// The K trees advance level by level together, so their latencies overlap;
// each value's summation order is the fixed tree order.
template <int K>
__device__ __forceinline__ void warp_df_reduce(DF (&v)[K]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        DF t[K];
#pragma unroll
        for (int k = 0; k < K; ++k) t[k] = df_shfl_down(v[k], o);
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = df_add(v[k], t[k]);
    }
}

// Block sum of K float values per thread for blocks of exactly NT threads:
// the values are transposed through shared memory, so that each warp sums
// only its share of the K values (NT/32 elements per lane, then one
// double-float shuffle tree per value, the trees advancing together) instead
// of every warp reducing all K and one warp reducing the warps' results.
// Fixed order, so deterministic.  Writes partials like block_partials_f.
template <int K, int NT>
__device__ __forceinline__ void block_partials_ft(float (&vf)[K], double* partials,
                                                  unsigned int G, unsigned int slot) {
    static_assert(NT % 32 == 0 && NT >= 32 && NT <= 1024, "whole warps");
    constexpr int NW = NT / 32, KW = (K + NW - 1) / NW;
    __shared__ float tr[K][NT];
#pragma unroll
    for (int k = 0; k < K; ++k) tr[k][threadIdx.x] = vf[k];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    DF v[KW];
#pragma unroll
    for (int i = 0; i < KW; ++i) {
        const int k = warp + i * NW;
        v[i] = DF{0.0f, 0.0f};
        if (k < K) {
            v[i] = DF{tr[k][lane], 0.0f};
#pragma unroll
            for (int j = 1; j < NW; ++j) v[i] = df_add(v[i], DF{tr[k][lane + 32 * j], 0.0f});
        }
    }
    warp_df_reduce<KW>(v);
    if (lane == 0) {
        float2* part = reinterpret_cast<float2*>(partials);
#pragma unroll
        for (int i = 0; i < KW; ++i) {
            const int k = warp + i * NW;
            if (k < K) part[(size_t)k * G + slot] = make_float2(v[i].hi, v[i].lo);
        }
    }
}

// Block sum of K float values in double-float (TwoSum) arithmetic, written
// value-major as partials[k * G + blockIdx.x] (float2 hi/lo); G = number of
// partial slots per value (the grid size).  All threads must call it.  Any
// block size: every warp reduces all K values, then warp 0 the warps' sums.
template <int K>
__device__ __forceinline__ void block_partials_fg(float (&vf)[K], double* partials,
                                                  unsigned int G, unsigned int slot) {
    __shared__ float2 red_p[K * 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    DF v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = DF{vf[k], 0.0f};
    warp_df_reduce<K>(v);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) red_p[k * 32 + warp] = make_float2(v[k].hi, v[k].lo);
    }
    __syncthreads();
    float2* part = reinterpret_cast<float2*>(partials);
    if (warp == 0) {
        DF t[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float2 x = lane < nw ? red_p[k * 32 + lane] : make_float2(0.0f, 0.0f);
            t[k] = DF{x.x, x.y};
        }
        warp_df_reduce<K>(t);
        // value-major: the final pass's loads of one value are coalesced
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < K; ++k) part[(size_t)k * G + slot] = make_float2(t[k].hi, t[k].lo);
        }
    }
}

// block_partials_fg, or with NT > 0 (the block has exactly NT threads) the
// transposed form block_partials_ft, as long as its shared-memory transpose
// stays within 16 KB (many values fall back to the per-warp form).
template <int K, int NT = 0>
__device__ __forceinline__ void block_partials_f(float (&vf)[K], double* partials, unsigned int G,
                                                 unsigned int slot) {
    if constexpr (NT > 0 && (size_t)K * NT * sizeof(float) <= 16384)
        block_partials_ft<K, NT>(vf, partials, G, slot);
    else
        block_partials_fg<K>(vf, partials, G, slot);
}
// the block's own slot: blockIdx.x
template <int K, int NT = 0>
__device__ __forceinline__ void block_partials_f(float (&vf)[K], double* partials, unsigned int G) {
    block_partials_f<K, NT>(vf, partials, G, blockIdx.x);
}

// Sum of the G block partials of each of K values (written by
// block_partials_f) by one block, in a fixed order: out[k] (double).
// All threads of the block must call it; thread 0 writes out.
template <int K>
__device__ __forceinline__ void final_partials_f(const double* partials, unsigned int G,
                                                 double* out) {
    __shared__ float2 red_f[K * 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    const float2* part = reinterpret_cast<const float2*>(partials);
    DF acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = DF{0.0f, 0.0f};
    // two blocks' partials per thread and round trip
    const unsigned int step = 2u * blockDim.x;
    for (unsigned int b0 = threadIdx.x; b0 < G; b0 += step) {
        const unsigned int b1 = b0 + blockDim.x;
        float2 x0[K], x1[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            x0[k] = __ldcg(part + (size_t)k * G + b0);
            x1[k] = b1 < G ? __ldcg(part + (size_t)k * G + b1) : make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
            acc[k] = df_add(acc[k], DF{x0[k].x, x0[k].y});
            acc[k] = df_add(acc[k], DF{x1[k].x, x1[k].y});
        }
    }
    warp_df_reduce<K>(acc);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) red_f[k * 32 + warp] = make_float2(acc[k].hi, acc[k].lo);
    }
    __syncthreads();
    if (warp == 0) {
        DF t[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float2 x = lane < nw ? red_f[k * 32 + lane] : make_float2(0.0f, 0.0f);
            t[k] = DF{x.x, x.y};
        }
        warp_df_reduce<K>(t);
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < K; ++k) out[k] = (double)t[k].hi + (double)t[k].lo;
        }
    }
}

// Grid-wide deterministic sum of K float values per thread: block partials,
// then the last block to finish (ticket) sums them in a fixed order into
// out[0..K).  Returns true on thread 0 of that last block (out is final
// there); the ticket is reset for the next launch.
template <int K, int NT = 0>
__device__ __forceinline__ bool grid_reduce_store_f(float (&vf)[K], double* partials,
                                                    unsigned int* ticket, double* out) {
    __shared__ bool is_last;
    block_partials_f<K, NT>(vf, partials, gridDim.x);
    // the partials may come from several warps (the transposed form): each
    // writer fences, and the barrier puts every write before the ticket, so
    // that the last block never reads a slot its owner has not yet written
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int t = atomicAdd(ticket, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    final_partials_f<K>(partials, gridDim.x, out);
    if (threadIdx.x == 0) {
        *ticket = 0u;
        return true;
    }
    return false;
}

template <int K>
__device__ __forceinline__ void grid_reduce_store(double (&v)[K], double* partials,
                                                  unsigned int* ticket, double* out,
                                                  bool accumulate) {
    __shared__ double red[K * 32];
    __shared__ bool is_last;
    block_reduce<K>(v, red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) partials[(size_t)blockIdx.x * K + k] = v[k];
        __threadfence();
        unsigned int t = atomicAdd(ticket, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    for (unsigned int bI = threadIdx.x; bI < gridDim.x; bI += blockDim.x) {
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] += ((volatile double*)partials)[(size_t)bI * K + k];
    }
    __syncthreads();
    block_reduce<K>(acc, red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) out[k] = (accumulate ? out[k] : 0.0) + acc[k];
        *ticket = 0u;
    }
}

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
};

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

// Device-side box update (barostat): the same quantities as fill_box_state.
__device__ __forceinline__ void fill_box_state_dev(BoxState& s, double L0, double L1, double L2) {
    const double Ls[3] = {L0, L1, L2};
    s.V = L0 * L1 * L2;
    const double M = (double)s.n[0] * (double)s.n[1] * (double)s.n[2];
    s.dV = s.V * rcp_d(M);
    for (int d = 0; d < 3; ++d) {
        const double iL = rcp_d(Ls[d]);
        s.L[d] = Ls[d];
        s.Lf[d] = (float)Ls[d];
        const double ih = (double)s.n[d] * iL;
        s.ih_hi[d] = (float)ih;
        s.ih_lo[d] = (float)(ih - (double)s.ih_hi[d]);
        s.kf[d] = (float)(2.0 * 3.14159265358979323846 * iL);
    }
    s.inv_dV = (float)(M * rcp_d(s.V));
}

// CSVR scale factors (hymd/thermostat.py:167-219, Bussi-Parrinello 2008 form)
// from the per-group sums ws[4g..4g+3] = (sum v_x, sum v_y, sum v_z, sum v^2),
// run by one thread once the sums are final.  state[4g] = alpha,
// state[4g+1..3] = the group's centre-of-mass velocity, state[8+g] += work.
// The O(1) quantities have no cancellation and are formed in FP32 (FP64
// division and square root are long sequences on GB300's FP64 pipe).
__device__ __forceinline__ void csvr_update(const HpfCsvrArgs& a, const double* ws,
                                            const double* randoms, int* counter, double* state,
                                            int* err) {
    const int s = *counter;
    const bool ok = s >= 0 && s < a.n_steps;
    if (!ok) hpf_flag(err, HPF_ERR_INDEX);
    const bool act = !(a.every > 1 && (s + 1) % a.every != 0);
    for (int g = 0; g < a.n_groups; ++g) {
        state[4 * g] = 1.0;
        for (int d = 0; d < 3; ++d) state[4 * g + 1 + d] = 0.0;
        if (!act) continue;
        const float N = (float)a.count[g];
        const float iN = 1.0f / N;
        float com[3] = {0, 0, 0};
        double K;
        if (a.remove_com && N > 1) {
            for (int d = 0; d < 3; ++d) com[d] = (float)ws[4 * g + d] * iN;
            K = 0.5 * a.mass * (ws[4 * g + 3] - (double)N * (double)(com[0] * com[0] +
                                                                      com[1] * com[1] +
                                                                      com[2] * com[2]));
        } else {
            // without COM removal the reference uses the whole system's K
            K = 0.5 * a.mass * (ws[3] + (a.n_groups > 1 ? ws[7] : 0.0));
        }
        const float Kt = (float)(1.5 * a.gas_constant * a.count[g] * a.target_temperature);
        const float Nf = 3.0f * N;
        const float R = ok ? (float)randoms[(int64_t)s * a.stride + a.offset + 2 * g] : 0.0f;
        const float S = ok ? (float)randoms[(int64_t)s * a.stride + a.offset + 2 * g + 1] : Nf - 1.0f;
        const float c = (float)a.c;
        const float q = Kt / (Nf * (float)K);
        const float alpha2 = c + (1.0f - c) * (S + R * R) * q + 2.0f * R * sqrtf(c * (1.0f - c) * q);
        state[4 * g] = (double)sqrtf(alpha2);
        for (int d = 0; d < 3; ++d) state[4 * g + 1 + d] = (double)com[d];
        state[8 + g] += K * ((double)alpha2 - 1.0);  // thermostat work (config.thermostat_work)
    }
    if (a.advance) *counter = s + 1;
}

// Isotropic SCR step (hymd/barostat_scr.py:34-132) run by one thread once all
// sums are final.  The pressure components are added in FP64; with the k = 0
// densities mean_t = m_t N_t / V the field part of p0 + p1 reduces to
//   -W/V + A + (Q mean + b).mean = A/2 + (1/2 mc.Q.mc) / V^2 - c.
// `bonded` holds {E_bond, bond_pr[3], E_angle, angle_pr[3]}.  The box is kept
// in float32 values, as the reference's float32 box_size array.
__device__ __forceinline__ void scr_update(const HpfScrArgs& a, double sum_v2,
                                           const double* field, const double* bonded,
                                           const double* randoms, int* counter, BoxState* bs,
                                           const Functional* fun, double* state, int* err) {
    const int s = *counter;
    const bool ok = s >= 0 && s < a.n_steps;
    if (!ok) hpf_flag(err, HPF_ERR_INDEX);
    state[12] = 1.0;
    if (!(a.every > 1 && (s + 1) % a.every != 0)) {
        const double V = bs->V;
        const double iV = rcp_d(V);
        const double A = field[0];
        const double p_kin = (2.0 / 3.0) * iV * (0.5 * a.mass * sum_v2);
        const double p01 = 0.5 * A + a.half_mQm * iV * iV - fun->c;
        const double sig2 = 2.0 * fun->sigma2_half_d;
        double ptot[2];
        for (int d = 0; d < 2; ++d)
            ptot[d] = p_kin + p01 - sig2 * field[1 + d] + (bonded[1 + d] + bonded[5 + d]) * iV;
        // the reference averages p_tot[-3:-1], i.e. the x and y components
        const double P = 0.5 * (ptot[0] + ptot[1]) * 16.61;
        const float R = ok ? (float)randoms[(int64_t)s * a.stride] : 0.0f;
        const float itau = 1.0f / (float)a.tau_p;
        const float noise = sqrtf((float)(2.0 * a.n_b * a.gas_constant * a.target_temperature *
                                          a.beta * a.dt_outer * a.n_b * iV) * itau) * R;
        const float log_alpha =
            -(float)(a.n_b * a.dt_outer * a.beta) * itau * (float)(a.target_pressure - P) + noise;
        const double alpha = (double)expf(log_alpha / 3.0f);
        fill_box_state_dev(*bs, (double)(float)(bs->L[0] * alpha),
                           (double)(float)(bs->L[1] * alpha), (double)(float)(bs->L[2] * alpha));
        state[12] = alpha;
        state[13] = P;
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

// Warp + block reduction of K doubles; thread 0 returns the block totals.
template <int K>
__device__ __forceinline__ void block_reduce(double (&v)[K], double* smem /* K*32 */) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
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
        for (int k = 0; k < K; ++k) {
            double x = lane < nw ? smem[k * 32 + lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            v[k] = x;
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

// Deterministic grid-wide sum of FP32 per-thread values (a thread adds only a
// few terms) with compensated double-float arithmetic above the thread: warp,
// block and the last block's pass over the block partials (stored as (hi, lo)
// pairs) all run on the FP32 pipe -- GB300's FP64 pipe is a small fraction of
// its FP32 one, and FP64 shuffles/adds in every block were a visible share of
// short kernels.  out[k] = hi + lo in FP64.  Returns true on thread 0 of the
// last block, after out[] has been written (for a fused epilogue).
template <int K>
__device__ __forceinline__ bool grid_reduce_store_f(float (&vf)[K], double* partials,
                                                    unsigned int* ticket, double* out) {
    __shared__ float2 red[K * 32];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    DF v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        v[k] = DF{vf[k], 0.0f};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] = df_add(v[k], df_shfl_down(v[k], o));
        if (lane == 0) red[k * 32 + warp] = make_float2(v[k].hi, v[k].lo);
    }
    __syncthreads();
    float2* part = reinterpret_cast<float2*>(partials);
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float2 x = lane < nw ? red[k * 32 + lane] : make_float2(0.0f, 0.0f);
            DF s{x.x, x.y};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s = df_add(s, df_shfl_down(s, o));
            if (lane == 0) part[(size_t)blockIdx.x * K + k] = make_float2(s.hi, s.lo);
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int t = atomicAdd(ticket, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    DF acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = DF{0.0f, 0.0f};
    for (unsigned int bI = threadIdx.x; bI < gridDim.x; bI += blockDim.x) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float2 x = __ldcg(part + (size_t)bI * K + k);
            acc[k] = df_add(acc[k], DF{x.x, x.y});
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] = df_add(acc[k], df_shfl_down(acc[k], o));
        if (lane == 0) red[k * 32 + warp] = make_float2(acc[k].hi, acc[k].lo);
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float2 x = lane < nw ? red[k * 32 + lane] : make_float2(0.0f, 0.0f);
            DF s{x.x, x.y};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s = df_add(s, df_shfl_down(s, o));
            if (lane == 0) out[k] = (double)s.hi + (double)s.lo;
        }
    }
    if (threadIdx.x == 0) {
        *ticket = 0u;
        return true;
    }
    return false;
}

// Deterministic grid-wide sum: each block stores its K partials; the last
// block to finish (ticket) adds them -- thread j takes blocks j, j+B, ...,
// then a fixed tree -- and writes out[k] (overwrite or accumulate).  The
// order never depends on scheduling, and the ticket resets itself, so the
// pattern is graph-replay safe.
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

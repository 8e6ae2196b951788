// Velocity-Verlet / rRESPA integrator pieces of HyMD on GB300.
//
// Reference behaviour (paths inside the HyMD project):
//   integrate_velocity / integrate_position   hymd/integrator.py:9-73
//   outer kick, inner loop, wrap              hymd/main.py:802-887, 1143-1169
// Each reference call `v = v + 0.5 * dt * (F / m)` is one FP32 rounding of
// F/m and one of the update; the kernels repeat exactly those roundings so
// that trajectories follow the reference's FP32 arithmetic.
#include <math.h>

#include "hpf_internal.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxForces = 8;

struct ForceList {
    const float* f[kMaxForces];
    int n;
};

int grid_for(int64_t work) {
    int64_t g = (work + kThreads - 1) / kThreads;
    if (g < 1) g = 1;
    const int64_t cap = 152 * 16;
    return (int)(g < cap ? g : cap);
}

__global__ void k_kick(float* __restrict__ v, ForceList fl, int64_t n3, float m, float hdt) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n3;
         e += (int64_t)gridDim.x * blockDim.x) {
        float x = v[e];
        for (int q = 0; q < fl.n; ++q) x = x + hdt * (fl.f[q][e] / m);
        v[e] = x;
    }
}

// np.mod(x, L) for L > 0: fmod, shifted into [0, L) when negative.
__device__ __forceinline__ float wrap(float x, float L) {
    float m = fmodf(x, L);
    if (m < 0.0f) m += L;
    return m;
}

__global__ void k_inner(float* __restrict__ r, float* __restrict__ v, const float* __restrict__ fb,
                        const float* __restrict__ fa, const float* __restrict__ fd, int64_t n,
                        float m, float hdt, float dt, int kicks, int drift,
                        const double* __restrict__ box) {
    const bool wrap_ = box != nullptr;
    const float L[3] = {wrap_ ? (float)box[0] : 0.f, wrap_ ? (float)box[1] : 0.f,
                        wrap_ ? (float)box[2] : 0.f};
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 3 * n;
         e += (int64_t)gridDim.x * blockDim.x) {
        float f = 0.0f;
        if (fb) f = fb[e];
        if (fa) f = f + fa[e];
        if (fd) f = f + fd[e];
        const float acc = f / m;
        float x = v[e];
        for (int q = 0; q < kicks; ++q) x = x + hdt * acc;
        v[e] = x;
        if (drift) {
            const float y = r[e] + dt * x;
            r[e] = wrap_ ? wrap(y, L[e % 3]) : y;
        }
    }
}

__global__ void k_sum_v2(const float* __restrict__ v, int64_t n3, double* out) {
    double acc[1] = {0.0};
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n3;
         e += (int64_t)gridDim.x * blockDim.x) {
        const double x = (double)v[e];
        acc[0] += x * x;
    }
    grid_reduce_store<1>(acc, ws_partials(out), ws_ticket(out), out, false);
}

// sum_e x[e] (y == NULL) or sum_e x[e] * y[e], accumulated in FP64
__global__ void k_sum_dot(const float* __restrict__ x, const float* __restrict__ y, int64_t n,
                          double* out) {
    double acc[1] = {0.0};
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x)
        acc[0] += y ? (double)x[e] * (double)y[e] : (double)x[e];
    grid_reduce_store<1>(acc, ws_partials(out), ws_ticket(out), out, false);
}

// ------------------------------------------------ thermostat / barostat ---
// Per-group sums of v (3) and v^2 for up to two coupling groups (FP64).
__global__ void k_group_sums(const float* __restrict__ v, const int32_t* __restrict__ group,
                             int64_t n, double* ws) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int g = group ? group[i] : 0;
        if (g < 0 || g > 1) continue;
        const double x = v[3 * i], y = v[3 * i + 1], z = v[3 * i + 2];
        acc[4 * g + 0] += x;
        acc[4 * g + 1] += y;
        acc[4 * g + 2] += z;
        acc[4 * g + 3] += x * x + y * y + z * z;
    }
    grid_reduce_store<8>(acc, ws_partials(ws), ws_ticket(ws), ws, false);
}

// CSVR (hymd/thermostat.py:111-219, Bussi-Parrinello 2008 form) scale factor
// of each group from its kinetic energy with the centre-of-mass motion
// removed.  randoms[step * stride + offset + 2g] = R, [.. + 1] = chi^2_{Nf-1}.
__global__ void k_csvr_alpha(const double* ws, HpfCsvrArgs a, const double* __restrict__ randoms,
                             int* counter, double* state, int* err) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int s = *counter;
    const bool ok = s >= 0 && s < a.n_steps;
    if (!ok) hpf_flag(err, HPF_ERR_INDEX);
    if (a.every > 1 && (s + 1) % a.every != 0) {
        for (int g = 0; g < a.n_groups; ++g) {
            state[4 * g] = 1.0;
            for (int d = 0; d < 3; ++d) state[4 * g + 1 + d] = 0.0;
        }
        if (a.advance) *counter = s + 1;
        return;
    }
    for (int g = 0; g < a.n_groups; ++g) {
        const double N = a.count[g];
        double com[3] = {0, 0, 0}, K;
        if (a.remove_com && N > 1) {
            for (int d = 0; d < 3; ++d) com[d] = ws[4 * g + d] / N;
            K = 0.5 * a.mass * (ws[4 * g + 3] - N * (com[0] * com[0] + com[1] * com[1] + com[2] * com[2]));
        } else {
            // without COM removal the reference uses the whole system's K
            K = 0.5 * a.mass * (ws[3] + (a.n_groups > 1 ? ws[7] : 0.0));
        }
        const double Kt = 1.5 * a.gas_constant * N * a.target_temperature;
        const double Nf = 3.0 * N;
        const double R = ok ? randoms[(int64_t)s * a.stride + a.offset + 2 * g] : 0.0;
        const double S = ok ? randoms[(int64_t)s * a.stride + a.offset + 2 * g + 1] : Nf - 1.0;
        const double c = a.c;
        double alpha2 = c + (1.0 - c) * (S + R * R) * Kt / (Nf * K) +
                        2.0 * R * sqrt(c * (1.0 - c) * Kt / (Nf * K));
        state[4 * g + 0] = sqrt(alpha2);
        for (int d = 0; d < 3; ++d) state[4 * g + 1 + d] = com[d];
        state[8 + g] += K * (alpha2 - 1.0);  // thermostat work (config.thermostat_work)
    }
    if (a.advance) *counter = s + 1;
}

__global__ void k_csvr_scale(float* __restrict__ v, const int32_t* __restrict__ group, int64_t n,
                             const double* __restrict__ state, int remove_com) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int g = group ? group[i] : 0;
        if (g < 0 || g > 1) continue;
        const float al = (float)state[4 * g];
        for (int d = 0; d < 3; ++d) {
            if (remove_com) {
                const float c = (float)state[4 * g + 1 + d];
                v[3 * i + d] = (v[3 * i + d] - c) * al + c;
            } else {
                v[3 * i + d] = v[3 * i + d] * al;
            }
        }
    }
}

// SCR isotropic barostat (hymd/barostat_scr.py:34-132): pressure from the
// FP64 field sums of the last field evaluation, the bonded virials of the
// last inner step and the current kinetic energy; scale box and positions.
__global__ void k_scr_iso(const double* __restrict__ vsum, const double* __restrict__ field,
                          const double* __restrict__ bonded, HpfScrArgs a,
                          const double* __restrict__ randoms, int* counter, BoxState* bs,
                          const Functional* __restrict__ fun, double* state, int* err) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int s = *counter;
    const bool ok = s >= 0 && s < a.n_steps;
    if (!ok) hpf_flag(err, HPF_ERR_INDEX);
    if (a.every > 1 && (s + 1) % a.every != 0) {
        state[12] = 1.0;
        if (a.advance) *counter = s + 1;
        return;
    }
    const double V = bs->V;
    const int T = a.n_types;
    double mean[HPF_MAX_TYPES];
    for (int t = 0; t < T; ++t) mean[t] = a.mass_count[t] / V;  // exact k = 0 densities
    double w0 = fun->c, p1dc = 0.0;
    for (int t = 0; t < T; ++t) {
        double u = fun->bd[t];
        for (int j = 0; j < T; ++j) u += fun->Qd[t * T + j] * mean[j];
        w0 += fun->bd[t] * mean[t] + 0.5 * (u - fun->bd[t]) * mean[t];
        p1dc += u * mean[t];
    }
    const double A = field[0];
    const double W = V * w0 + 0.5 * V * A;
    const double ke = 0.5 * a.mass * vsum[0];
    const double p_kin = 2.0 / (3.0 * V) * ke;
    const double p0 = -W / V;
    const double p1 = A + p1dc;
    const double sig2 = 2.0 * fun->sigma2_half_d;
    double ptot[3];
    for (int d = 0; d < 3; ++d)
        ptot[d] = p_kin + p0 + p1 - sig2 * field[1 + d] + bonded[1 + d] / V + bonded[5 + d] / V;
    // the reference averages p_tot[-3:-1], i.e. the x and y components
    const double P = 0.5 * (ptot[0] + ptot[1]) * 16.61;
    const double R = ok ? randoms[(int64_t)s * a.stride] : 0.0;
    const double noise = sqrt(2.0 * a.n_b * a.gas_constant * a.target_temperature * a.beta *
                              a.dt_outer * a.n_b / (V * a.tau_p)) * R;
    const double log_alpha = -a.n_b * a.dt_outer * a.beta / a.tau_p * (a.target_pressure - P) + noise;
    const double alpha = exp(log_alpha / 3.0);
    // the reference keeps the box in float32
    const double L0 = (double)(float)(bs->L[0] * alpha);
    const double L1 = (double)(float)(bs->L[1] * alpha);
    const double L2 = (double)(float)(bs->L[2] * alpha);
    const int nn[3] = {bs->n[0], bs->n[1], bs->n[2]};
    fill_box_state(*bs, L0, L1, L2, nn);
    state[12] = alpha;
    state[13] = P;
    if (a.advance) *counter = s + 1;
}

__global__ void k_scale_positions(float* __restrict__ r, int64_t n3, const double* __restrict__ state) {
    const float al = (float)state[12];
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n3;
         e += (int64_t)gridDim.x * blockDim.x)
        r[e] = r[e] * al;
}

}  // namespace

extern "C" {

int hpf_csvr(float* v, const int32_t* group, int64_t n, const HpfCsvrArgs* args,
             const double* randoms, int* counter, double* state, double* ws, int* d_err,
             void* stream) {
    if (!v || n < 0 || !args || !randoms || !counter || !state || !ws) return HPF_ERR_ARG;
    if (args->n_groups < 1 || args->n_groups > 2 || (args->n_groups > 1 && !group))
        return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    int64_t g = (n + kThreads - 1) / kThreads;
    g = g < 1 ? 1 : (g > HPF_REDUCE_BLOCKS ? HPF_REDUCE_BLOCKS : g);
    k_group_sums<<<(int)g, kThreads, 0, st>>>(v, group, n, ws);
    HPF_LAUNCH_CHECK();
    k_csvr_alpha<<<1, 32, 0, st>>>(ws, *args, randoms, counter, state, d_err);
    HPF_LAUNCH_CHECK();
    k_csvr_scale<<<grid_for(n), kThreads, 0, st>>>(v, group, n, state, args->remove_com);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_scr_isotropic(hpf_ctx* ctx, float* r, const float* v, int64_t n,
                      const double* field_sums, const double* bonded_out,
                      const HpfScrArgs* args, const double* randoms, int* counter,
                      double* state, double* ws, int* d_err, void* stream) {
    if (!ctx || !r || !v || n < 0 || !field_sums || !bonded_out || !args || !randoms ||
        !counter || !state || !ws || args->n_types != ctx->T)
        return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    int64_t g = (3 * n + kThreads - 1) / kThreads;
    g = g < 1 ? 1 : (g > HPF_REDUCE_BLOCKS ? HPF_REDUCE_BLOCKS : g);
    k_sum_v2<<<(int)g, kThreads, 0, st>>>(v, 3 * n, ws);
    HPF_LAUNCH_CHECK();
    k_scr_iso<<<1, 32, 0, st>>>(ws, field_sums, bonded_out, *args, randoms, counter, ctx->d_box,
                                ctx->d_fun, state, d_err);
    HPF_LAUNCH_CHECK();
    k_scale_positions<<<grid_for(3 * n), kThreads, 0, st>>>(r, 3 * n, state);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_sum_dot(const float* x, const float* y, int64_t n, double* out, void* stream) {
    if (!x || !out || n < 0) return HPF_ERR_ARG;
    int64_t g = (n + kThreads - 1) / kThreads;
    if (g < 1) g = 1;
    if (g > HPF_REDUCE_BLOCKS) g = HPF_REDUCE_BLOCKS;
    k_sum_dot<<<(int)g, kThreads, 0, as_stream(stream)>>>(x, y, n, out);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_kick(float* v, const float* const* forces, int n_f, int64_t n, double mass, double dt,
             void* stream) {
    if (!v || n < 0 || n_f < 0 || n_f > kMaxForces || (n_f > 0 && !forces) || !(mass > 0))
        return HPF_ERR_ARG;
    if (n == 0 || n_f == 0) return HPF_OK;
    ForceList fl;
    fl.n = n_f;
    for (int q = 0; q < n_f; ++q) {
        if (!forces[q]) return HPF_ERR_ARG;
        fl.f[q] = forces[q];
    }
    k_kick<<<grid_for(3 * n), kThreads, 0, as_stream(stream)>>>(v, fl, 3 * n, (float)mass,
                                                                (float)(0.5 * dt));
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_inner_kick_drift(float* r, float* v, const float* fb, const float* fa, const float* fd,
                         int64_t n, double mass, double dt, int kicks, int drift,
                         const double* box, void* stream) {
    if (!v || n < 0 || kicks < 0 || !(mass > 0) || (drift && !r)) return HPF_ERR_ARG;
    if (n == 0) return HPF_OK;
    k_inner<<<grid_for(3 * n), kThreads, 0, as_stream(stream)>>>(
        r, v, fb, fa, fd, n, (float)mass, (float)(0.5 * dt), (float)dt, kicks, drift, box);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_sum_v2(const float* v, int64_t n, double* out, void* stream) {
    if (!v || !out || n < 0) return HPF_ERR_ARG;
    int64_t g = (3 * n + kThreads - 1) / kThreads;
    if (g < 1) g = 1;
    if (g > HPF_REDUCE_BLOCKS) g = HPF_REDUCE_BLOCKS;
    k_sum_v2<<<(int)g, kThreads, 0, as_stream(stream)>>>(v, 3 * n, out);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

}  // extern "C"

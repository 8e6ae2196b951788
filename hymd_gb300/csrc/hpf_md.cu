// Velocity-Verlet / rRESPA integrator pieces, CSVR thermostat and SCR
// barostat of HyMD on GB300.
//
// Reference behaviour (paths inside the HyMD project):
//   integrate_velocity / integrate_position   hymd/integrator.py:9-73
//   outer kick, inner loop, wrap              hymd/main.py:802-887, 1143-1169
//   csvr_thermostat                           hymd/thermostat.py:111-219
//   SCR barostat, isotropic / semi-isotropic  hymd/barostat_scr.py:34-132, :133-284
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

int reduce_grid_md(int64_t work) {
    int64_t g = (work + kThreads - 1) / kThreads;
    g = g < 1 ? 1 : (g > HPF_REDUCE_GRID ? HPF_REDUCE_GRID : g);
    return (int)g;
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
    float acc[1] = {0.0f};
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n3;
         e += (int64_t)gridDim.x * blockDim.x)
        acc[0] = fmaf(v[e], v[e], acc[0]);
    grid_reduce_store_f<1, kThreads>(acc, ws_partials(out), ws_ticket(out), out);
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

// ------------------------------------------------------------ thermostat ---
// Per-group sums of v (3) and v^2 for up to two coupling groups; the last
// block then forms each group's CSVR scale factor (Bussi-Parrinello 2008
// form, hymd/thermostat.py:167-219) from the kinetic energy with the
// centre-of-mass motion removed.  randoms[step * stride + offset + 2g] = R,
// [.. + 1] = chi^2_{Nf-1}.
// The preceding outer half kick v += 0.5 dt_o F_q/m (forces in `kick`) is
// applied first, in the same pass.
__global__ void k_csvr_sums_alpha(float* __restrict__ v, const int32_t* __restrict__ group,
                                  int64_t n, ForceList kick, float kick_h, double* ws,
                                  HpfCsvrArgs a, const double* __restrict__ randoms, int* counter,
                                  double* state, int* err) {
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const float m = (float)a.mass;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float w[3];
        for (int d = 0; d < 3; ++d) {
            float x = v[3 * i + d];
            for (int q = 0; q < kick.n; ++q) x = x + kick_h * (kick.f[q][3 * i + d] / m);
            w[d] = x;
            if (kick.n) v[3 * i + d] = x;
        }
        const int g = group ? group[i] : 0;
        if (g < 0 || g > 1) continue;
        const float x = w[0], y = w[1], z = w[2];
        acc[4 * g + 0] += x;
        acc[4 * g + 1] += y;
        acc[4 * g + 2] += z;
        acc[4 * g + 3] += fmaf(x, x, fmaf(y, y, z * z));
    }
    if (!grid_reduce_store_f<8, kThreads>(acc, ws_partials(ws), ws_ticket(ws), ws)) return;
    csvr_update(a, ws, randoms, counter, state, err);
}

// v <- A_g v + B_g with the composed per-group transform csvr_update leaves
// in state (the reference's group-by-group rescaling, thermostat.py:190-219).
// `remove_com` is carried by the transform and not read here.
__global__ void k_csvr_scale(float* __restrict__ v, const int32_t* __restrict__ group, int64_t n,
                             const double* __restrict__ state, int remove_com) {
    (void)remove_com;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int g = group ? group[i] : 0;
        if (g < 0 || g > 1) continue;
        const float al = (float)state[4 * g];
        for (int d = 0; d < 3; ++d)
            v[3 * i + d] = fmaf(al, v[3 * i + d], (float)state[4 * g + 1 + d]);
    }
}

// One coupling group (no group array): the same v <- A v + B_d as
// k_csvr_scale over the flat array of 3n floats, four per thread as one
// 16-byte access (v must be 16-byte aligned); the component of flat element
// j is j mod 3.  Bit-equal to k_csvr_scale.
__global__ void k_csvr_scale_flat(float* __restrict__ v, int64_t n3,
                                  const double* __restrict__ state) {
    pdl_wait();
    const float al = (float)state[0];
    const float b0 = (float)state[1], b1 = (float)state[2], b2 = (float)state[3];
    const int64_t n4 = n3 >> 2;
    float4* v4 = reinterpret_cast<float4*>(v);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n4; k += stride) {
        float4 x = v4[k];
        const int d = (int)((4 * k) % 3);  // components d, d+1, d+2, d of the four
        const float bd = d == 0 ? b0 : (d == 1 ? b1 : b2);
        const float be = d == 0 ? b1 : (d == 1 ? b2 : b0);
        const float bf = d == 0 ? b2 : (d == 1 ? b0 : b1);
        x.x = fmaf(al, x.x, bd);
        x.y = fmaf(al, x.y, be);
        x.z = fmaf(al, x.z, bf);
        x.w = fmaf(al, x.w, bd);
        v4[k] = x;
    }
    for (int64_t j = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n3; j += stride) {
        const int d = (int)(j % 3);
        v[j] = fmaf(al, v[j], d == 0 ? b0 : (d == 1 ? b1 : b2));
    }
}

void launch_csvr_scale(float* v, const int32_t* group, int64_t n, const double* state,
                       int remove_com, cudaStream_t st) {
    if (!group && (reinterpret_cast<uintptr_t>(v) & 15) == 0) {
        const int64_t n4 = (3 * n + 3) / 4;
        // a failed launch is left in the runtime's last error for the caller's check
        (void)launch_pdl(k_csvr_scale_flat, grid_for(n4), kThreads, 0, st, v, 3 * n, state);
    } else {
        k_csvr_scale<<<grid_for(n), kThreads, 0, st>>>(v, group, n, state, remove_com);
    }
}

// -------------------------------------------------------------- barostat ---
// Sum of v^2, then (last block) the isotropic SCR step: pressure from the
// field sums of the last field evaluation, the bonded virials of the last
// inner step and the kinetic energy; box scaled by alpha (kept in float32
// values, as the reference's float32 box_size array).  With the k = 0
// densities mean_t = m_t N_t / V the field part of p0 + p1 reduces to
//   -W/V + A + (Q mean + b).mean = A/2 + (1/2 mc.Q.mc) / V^2 - c.
__global__ void k_scr_sums_alpha(const float* __restrict__ v, int64_t n3, double* ws,
                                 const double* __restrict__ field,
                                 const double* __restrict__ bonded, HpfScrArgs a,
                                 const double* __restrict__ randoms, int* counter, BoxState* bs,
                                 const Functional* __restrict__ fun, double* state, int* err) {
    float acc[1] = {0.0f};
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n3;
         e += (int64_t)gridDim.x * blockDim.x)
        acc[0] = fmaf(v[e], v[e], acc[0]);
    if (!grid_reduce_store_f<1, kThreads>(acc, ws_partials(ws), ws_ticket(ws), ws)) return;
    scr_update(a, ws[0], field, bonded, randoms, counter, bs, fun, state, err);
}

__global__ void k_scale_positions(float* __restrict__ r, int64_t n3, const double* __restrict__ state) {
    const float al = (float)state[12];
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n3;
         e += (int64_t)gridDim.x * blockDim.x)
        r[e] = r[e] * al;
}

// Semi-isotropic position update as the reference performs it
// (hymd/barostat_scr.py:249, :280): `positions[:][0:2] *= alpha_L` and
// `positions[:][2] *= alpha_N` index ROWS, so all three coordinates of
// particles 0 and 1 are scaled by alpha_L and those of particle 2 by
// alpha_N; every other particle keeps its coordinates.  float32 values times
// a float64 factor, rounded back to float32.
__global__ void k_scale_positions_semi(float* __restrict__ r, int64_t n,
                                       const double* __restrict__ state) {
    const int e = threadIdx.x;  // one block of 9 threads
    const int p = e / 3;
    if (e >= 9 || p >= n) return;
    const double al = p < 2 ? state[12] : state[14];
    r[e] = (float)((double)r[e] * al);
}

}  // namespace

extern "C" {

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

int hpf_csvr(float* v, const int32_t* group, int64_t n, const float* const* kick_forces,
             int n_kick, double kick_dt, const HpfCsvrArgs* args, const double* randoms,
             int* counter, double* state, double* ws, int* d_err, void* stream) {
    if (!v || n < 0 || !args || !randoms || !counter || !state || !ws || n_kick < 0 ||
        n_kick > kMaxForces || (n_kick > 0 && !kick_forces))
        return HPF_ERR_ARG;
    if (args->n_groups < 1 || args->n_groups > 2 || (args->n_groups > 1 && !group))
        return HPF_ERR_ARG;
    ForceList fl;
    fl.n = n_kick;
    for (int q = 0; q < n_kick; ++q) {
        if (!kick_forces[q]) return HPF_ERR_ARG;
        fl.f[q] = kick_forces[q];
    }
    cudaStream_t st = as_stream(stream);
    k_csvr_sums_alpha<<<reduce_grid_md(n), kThreads, 0, st>>>(
        v, group, n, fl, (float)(0.5 * kick_dt), ws, *args, randoms, counter, state, d_err);
    HPF_LAUNCH_CHECK();
    launch_csvr_scale(v, group, n, state, args->remove_com, st);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_csvr_scale(float* v, const int32_t* group, int64_t n, const double* state,
                   int remove_com, void* stream) {
    if (!v || !state || n < 0) return HPF_ERR_ARG;
    if (n == 0) return HPF_OK;
    launch_csvr_scale(v, group, n, state, remove_com, as_stream(stream));
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_scr_scale_positions(float* r, int64_t n, const double* state, int mode, void* stream);

int hpf_scr_isotropic(hpf_ctx* ctx, float* r, const float* v, int64_t n,
                      const double* field_sums, const double* bonded_out,
                      const HpfScrArgs* args, const double* randoms, int* counter,
                      double* state, double* ws, int* d_err, void* stream) {
    if (!ctx || !r || !v || n < 0 || !field_sums || !bonded_out || !args || !randoms ||
        !counter || !state || !ws || args->n_types != ctx->T)
        return HPF_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    k_scr_sums_alpha<<<reduce_grid_md(3 * n), kThreads, 0, st>>>(
        v, 3 * n, ws, field_sums, bonded_out, *args, randoms, counter, ctx->d_box, ctx->d_fun,
        state, d_err);
    HPF_LAUNCH_CHECK();
    return hpf_scr_scale_positions(r, n, state, args->mode, stream);
}

int hpf_scr_scale_positions(float* r, int64_t n, const double* state, int mode, void* stream) {
    if (!r || !state || n < 0 || mode < 0 || mode > 1) return HPF_ERR_ARG;
    if (n == 0) return HPF_OK;
    cudaStream_t st = as_stream(stream);
    if (mode == 0)
        k_scale_positions<<<grid_for(3 * n), kThreads, 0, st>>>(r, 3 * n, state);
    else
        k_scale_positions_semi<<<1, 9, 0, st>>>(r, n, state);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_sum_dot(const float* x, const float* y, int64_t n, double* out, void* stream) {
    if (!x || !out || n < 0) return HPF_ERR_ARG;
    k_sum_dot<<<reduce_grid_md(n), kThreads, 0, as_stream(stream)>>>(x, y, n, out);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

int hpf_sum_v2(const float* v, int64_t n, double* out, void* stream) {
    if (!v || !out || n < 0) return HPF_ERR_ARG;
    k_sum_v2<<<reduce_grid_md(3 * n), kThreads, 0, as_stream(stream)>>>(v, 3 * n, out);
    HPF_LAUNCH_CHECK();
    return HPF_OK;
}

}  // extern "C"

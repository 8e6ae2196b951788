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

}  // namespace

extern "C" {

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

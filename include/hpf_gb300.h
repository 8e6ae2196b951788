/*
 * hpf_gb300 -- C ABI of the GB300 (sm_103a) hybrid particle-field force path.
 *
 * Every entry point takes raw device pointers, element counts and a CUDA
 * stream (as void*), returns an int status (HPF_OK = 0) and throws nothing.
 * Scalars that a kernel produces (energies, virials) are written to
 * caller-provided DEVICE buffers, so no entry point synchronises the stream
 * unless its comment says so; all of them can be captured in a CUDA graph
 * except hpf_ctx_create/destroy/set_* and hpf_get_error.
 *
 * Array conventions (all row-major, device memory):
 *   positions, velocities, forces   float[N][3]
 *   types                           int32[N]      (0 <= type < n_types)
 *   real mesh                       float[n0][n1][n2]        (M = n0*n1*n2)
 *   half spectrum                   float2[n0][n1][n2/2+1]   (Mc points)
 *   per-type stacks                 float[T][M] / float2[T][Mc]
 *   force-mesh stack                float[T][3][M]
 * Spectra follow the reference mesh library's convention: r2c is normalised
 * by 1/M and c2r is unnormalised.
 *
 * Each declaration names the reference function it replaces (paths inside the
 * HyMD project).
 */
#ifndef HPF_GB300_H
#define HPF_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    HPF_OK = 0,
    HPF_ERR_ARG = 1,          /* bad argument (null pointer, size, shape)        */
    HPF_ERR_CUDA = 2,         /* a CUDA runtime call failed                      */
    HPF_ERR_CUFFT = 3,        /* a cuFFT call failed                             */
    HPF_ERR_INDEX = 4,        /* device saw a particle/type index out of range   */
    HPF_ERR_NONFINITE = 5,    /* device saw a non-finite position                */
    HPF_ERR_TIMEOUT = 6,      /* a bounded device wait ran out                   */
    HPF_ERR_NOT_IMPLEMENTED = 7,
    HPF_ERR_SCRATCH_LIMIT = 8 /* request exceeds a fixed-size static scratch     */
};

typedef struct hpf_ctx hpf_ctx; /* mesh context: geometry, cuFFT plans, scratch */

/* Reductions are deterministic: every block stores its partial sums, the
 * last block adds them in block order.  Entry points without a context
 * (bonded, integrator) take a caller-owned device workspace `out` of
 * HPF_OUT_DOUBLES doubles: out[0..7] are the results, the rest holds the
 * block partials and a self-resetting ticket.  Zero it once before first use. */
#define HPF_REDUCE_BLOCKS 1024
#define HPF_OUT_DOUBLES (8 + 8 * HPF_REDUCE_BLOCKS + 8)

/* ---- thermostat / barostat on the device -----------------------------------
 * The random numbers are drawn on the host in the reference's order (numpy
 * Generator: barostat normal(), then per thermostat group normal() and
 * chisquare(N_f - 1)) into a device table with one row per outer step; a
 * device step counter selects the row, so captured graphs replay them. */
typedef struct {
    int n_groups;       /* coupling groups, 1 or 2 (group ids from `group`)      */
    int remove_com;     /* remove / restore each group's centre-of-mass velocity */
    int n_steps;        /* rows in the random table                              */
    int stride;         /* doubles per row                                       */
    int offset;         /* row[offset + 2g] = R, row[offset + 2g + 1] = chi^2    */
    int advance;        /* increment the step counter afterwards                 */
    int every;          /* act when (step + 1) % every == 0 (n_b)                */
    int pad;
    double count[2];    /* particles per group                                   */
    double mass, gas_constant, target_temperature;
    double c;           /* exp(-dt_outer / tau)                                  */
} HpfCsvrArgs;

/* SCR barostat (hymd/barostat_scr.py).  mode 0: isotropic (:34-132), one
 * normal() per barostat step at row[0]; mode 1: semi-isotropic with z normal
 * (:133-284), normal() for the lateral then the normal direction at row[0]
 * and row[1]; a direction is coupled when its target pressure is nonzero
 * (couple_l / couple_n, the reference's truth test of P_L / P_N). */
typedef struct {
    int n_types, n_steps, stride, advance;
    int every;
    int mode;               /* 0 isotropic, 1 semi-isotropic                     */
    int couple_l, couple_n; /* semi-isotropic: lateral / normal directions coupled */
    double half_mQm;        /* 1/2 mc.Q.mc with mc_t = m_t N_t (paint mass x count),
                               so the k = 0 densities are mc_t / V               */
    double mass, gas_constant, target_temperature;
    double target_pressure; /* bar (semi-isotropic: lateral P_L)                */
    double beta;            /* isothermal compressibility (1/bar)               */
    double tau_p, dt_outer, n_b;
    double target_pressure_n; /* bar, semi-isotropic normal P_N                 */
} HpfScrArgs;

/* Optional outer half kick fused into the last readout of a field
 * evaluation (hymd/main.py:1143-1169): v += 0.5 dt_outer F/mass for each of
 * the n_prev slow forces already computed (in order), then for the force
 * this readout produces.  With thermo != NULL the same pass accumulates the
 * per-group velocity sums and the grid's last block forms the CSVR scale
 * factors (as hpf_csvr does, without applying them: call hpf_csvr_scale). */
typedef struct {
    float* v;
    const float* prev[4];
    int n_prev;
    int pad;
    double mass, dt_outer;
    const HpfCsvrArgs* thermo;
    const int32_t* group;
    const double* randoms;
    int* counter;
    double* state;
    double* ws;     /* reduction workspace (HPF_OUT_DOUBLES) */
    int* d_err;
} HpfKick;

/* ---- context ------------------------------------------------------------
 * Replaces initialize_pm (hymd/field.py:10-149): builds the mesh geometry and
 * the cuFFT plans for n_types densities.  Allocates the paint accumulators,
 * the box state and the cuFFT work area on the current device.               */
int hpf_ctx_create(hpf_ctx** out, int n0, int n1, int n2, int n_types, const double box[3]);
int hpf_ctx_destroy(hpf_ctx* ctx);
/* Box change (barostat rescale, hymd/barostat_scr.py:131): rewrites the
 * device box state; plans are kept.  Stream-ordered. */
int hpf_ctx_set_box(hpf_ctx* ctx, const double box[3], void* stream);
/* Device pointer to the box state (double L[3], V, dV at offsets 0..4). */
int hpf_ctx_box_state(hpf_ctx* ctx, void** d_state);
/* Transform path of hpf_field_step and hpf_pic_step (same arithmetic, FP32
 * either way): on a mesh with n0 a power of two in 8..256 or one of 24, 48,
 * 96, 192, and (n1, n2) both powers of two in 16..128 or n1 = n2 in {24, 48,
 * 96} (n_types <= 8), the default is this library's fused passes
 * (shared-memory FFTs, the k-space map inside the x transform, the paint's
 * accumulators read directly);
 * fused = 0 selects the cuFFT path.  fused = 1 on a mesh that does not
 * qualify returns HPF_ERR_ARG.  The getter reports the current choice and
 * whether the fused path is available (either pointer may be NULL). */
int hpf_ctx_set_spectral(hpf_ctx* ctx, int fused);
int hpf_ctx_get_spectral(const hpf_ctx* ctx, int* fused, int* available);
/* Column-tile width of the fused k-space pass (4, 8 or 16 (y, kz) columns
 * per block; the knob of the k-space autotuner, no counterpart in the
 * reference, whose transforms are pfft's).  The width changes the tiling and
 * the order of the energy/virial partial sums, not the force arithmetic.
 * The setter returns HPF_ERR_ARG for a width this mesh does not allow (or
 * without the fused path); allowed_mask gets the allowed widths OR'ed
 * together (0 without the fused path).  A graph captured before a change
 * keeps the width it was captured with. */
int hpf_ctx_set_spectral_tile(hpf_ctx* ctx, int width);
int hpf_ctx_get_spectral_tile(const hpf_ctx* ctx, int* width, int* allowed_mask);
/* Quadratic interaction functional w = 1/2 phi.Q.phi + b.phi + c and filter
 * width sigma (hymd/hamiltonian.py:74-486, H at :57-71).  Q is T*T row-major. */
int hpf_ctx_set_functional(hpf_ctx* ctx, const double* Q, const double* b, double c,
                           double sigma);
/* First error recorded by a device-side check since the last call; clears
 * it.  Synchronises the stream. */
int hpf_get_error(hpf_ctx* ctx, void* stream, int* code);
const char* hpf_status_string(int status);

/* ---- particle -> mesh ----------------------------------------------------
 * pm.paint(positions[types == t], mass=m[t]) / dV for every t
 * (hymd/field.py:573-575).  Deterministic CIC with 64-bit fixed-point
 * accumulation.  type_mass: host float[T].  phi_out: float[T][M].          */
int hpf_paint(hpf_ctx* ctx, const float* pos, const int32_t* types, int64_t n,
              const double* type_mass, float* phi_out, void* stream);
/* pm.paint(positions, mass=charges) / dV (hymd/field.py:363-364). */
int hpf_paint_charge(hpf_ctx* ctx, const float* pos, const float* charges, int64_t n,
                     float* rho_out, void* stream);

/* ---- transforms (cuFFT, FP32) --------------------------------------------
 * r2c / c2r of `batch` stacked grids (phi[t].r2c, phi_fourier[t].c2r). */
int hpf_r2c(hpf_ctx* ctx, const float* grids, void* spectra, int batch, void* stream);
int hpf_c2r(hpf_ctx* ctx, const void* spectra, float* grids, int batch, void* stream);

/* ---- fused k-space pass --------------------------------------------------
 * One pass over the half spectrum replacing field.py:576-616: from the raw
 * (unnormalised) r2c spectra of the T density grids it writes
 *   force_k[t][d] = -i k_d H(k) v_t(k),  v_t = H (Q phi~)_t + b_t delta_k0,
 *   phi~ = H phi / M
 * and, when the pointers are non-null, the filtered spectra phi_fourier[t]
 * = phi~ and the potential spectra v_k[t].  When sums != NULL it adds FP64
 * Parseval sums over k != 0 with half-spectrum weights:
 *   sums[0] = sum_k w_k sum_ij Q_ij Re(phi~_i conj phi~_j)
 *   sums[1+d] = sum_k w_k k_d^2 (same)            (d = 0, 1, 2)
 * (energy, p1 and the laplacian pressure term of hymd/pressure.py:84-121).
 * sums is a device double[4] that this call overwrites. */
int hpf_kspace_force(hpf_ctx* ctx, const void* phi_k_raw, void* force_k,
                     void* phi_fourier, void* v_k, double* sums, void* stream);
/* Parseval sums (as above) from already filtered spectra phi~[t] and, when
 * psi_k != NULL, the PIC cross terms with per-type charges (host float[T]):
 *   sums[4] = sum_k w_k sum_t q_t Re(psi conj phi~_t)   (k = 0 included)
 *   sums[5+d] = sum_k w_k k_d^2 sum_t q_t Re(psi conj phi~_t)
 * sums: device double[8]. */
int hpf_kspace_sums(hpf_ctx* ctx, const void* phi_fourier, const void* psi_k,
                    const double* type_charges, double* sums, void* stream);

/* FP64 energies and pressure sums of the current positions (the quantities
 * of compute_field_and_kinetic_energy, hymd/field.py:619-703, and of
 * comp_pressure, hymd/pressure.py:84-121).  The fixed-point densities (and,
 * when charges != NULL, the charge density) are converted to double grids,
 * transformed by an FP64 cuFFT and reduced in FP64 over the half spectrum.
 * out: device double[32]:
 *   out[0]    A   = sum_{k!=0} w_k sum_ij Q_ij Re(phi~_i conj phi~_j)
 *   out[1+d]  B_d = sum_{k!=0} w_k k_d^2 (same)
 *   out[4]    sum_k w_k Re(rho_k conj psi_k)   (W_elec = V/2 out[4] - E_self)
 *   out[5]    sum_k w_k sum_t q_t Re(psi_k conj phi~_t)   (type_charges q_t)
 *   out[6+d]  the same weighted by k_d^2
 *   out[16+t] mean of phi_t
 * so that W = V w(mean phi) + V/2 A.  Allocates its FP64 buffers and plan
 * on first use (not capturable then). */
int hpf_energy_fp64(hpf_ctx* ctx, const float* pos, const int32_t* types, int64_t n,
                    const double* type_mass, const float* charges, const double* type_charges,
                    double elec_factor, double* out, void* stream);

/* ---- reverse mode through the force ----------------------------------------
 * No counterpart in the reference (it has no gradients); used to
 * differentiate MD trajectories.  With the cotangent lam (device float[n][3])
 * of the field force F = compute_field_force after update_field
 * (hymd/field.py:152-200, 428-616) at positions pos:
 *   grad_pos (device float[n][3]) = d(lam . F)/dpos -- a local CIC-gradient
 *     readout of lam . E plus a global term through the lambda-weighted
 *     paint, the adjoint k-space operator and a CIC-gradient readout;
 *   dQ (device double[T][T], or NULL) = d(lam . F)/dQ_tj for the quadratic
 *     functional's matrix Q (hpf_ctx_set_functional).
 * The lambda paint uses FP32 atomics (not bit-reproducible).  T <= 8. */
int hpf_field_force_vjp(hpf_ctx* ctx, const float* pos, const int32_t* types, int64_t n,
                        const double* type_mass, const float* lam, float* grad_pos, double* dQ,
                        void* stream);
/* Vector-Jacobian product of the PIC_Spectral electrostatic force
 * (hymd/field.py:241-403: F_i = q_i E(x_i), E = -grad psi, psi = 4 pi f H
 * rho / k^2, f = elec_factor) with a cotangent lam (float[n][3]):
 * grad_pos (float[n][3]) = d(lam . F)/dx, the local term (q_i times the
 * CIC-gradient readout of lam_i . E) plus the global one (the
 * charge-weighted cotangent paint through the adjoint Poisson map, read out
 * with CIC-gradient weights times q_j / dV).  Charges are not differentiated.
 * Runs on cuFFT (plans created on first use, outside capture).  No
 * counterpart in the reference, which has no derivatives of the forces. */
int hpf_pic_force_vjp(hpf_ctx* ctx, const float* pos, const float* charges, int64_t n,
                      double elec_factor, const float* lam, float* grad_pos, void* stream);
/* out (device float[n][3]) = d/de F_b(r + e lam) at e = 0 for the bond and
 * angle forces of cbf / caf (the terms of hpf_bonds / hpf_angles): minus the
 * Hessian of the bonded energy times lam, which is also the vector-Jacobian
 * product of the forces (the Hessian is symmetric).  Forward-mode dual
 * arithmetic through the same FP32 formulas; out is zeroed first. */
int hpf_bonded_hvp(float* out, const float* r, const float* lam, int64_t n, const double* box,
                   const int32_t* ba, const int32_t* bb, const float* br0, const float* bk,
                   int64_t nb, const int32_t* aa, const int32_t* ab, const int32_t* ac,
                   const float* at0, const float* ak, int64_t na, int* d_err, void* stream);
/* Directional derivative of the four-body forces (compute_dihedral_forces.f90:
 * 61-134 with the CBT bending of dipole_reconstruction.f90:50-106; no
 * dipoles) along lam, ADDED to out (float[n][3]): minus the Hessian of the
 * dihedral energy times lam, the four-body part of the vector-Jacobian
 * product of reverse mode (hpf_bonded_hvp gives the bonds and angles and
 * zeroes out first).  Forward-mode dual arithmetic over the same expressions
 * as the force kernel; coeff float[nd][6][5], dtype / last int32[nd] as for
 * hpf_dihedrals.  No counterpart in the reference, which has no
 * derivatives of the forces. */
int hpf_dihedral_hvp(float* out, const float* r, const float* lam, int64_t n, const double* box,
                     const int32_t* a, const int32_t* b, const int32_t* c, const int32_t* d,
                     const float* coeff, const int32_t* dtype, const int32_t* last, int64_t nd,
                     int* d_err, void* stream);

/* ---- PIC_Spectral_GPE electrostatics ------------------------------------
 * update_field_force_q_GPE (hymd/field.py:764-1112) and the energy of
 * compute_field_energy_q_GPE (:706-761): dielectric
 * eps = sum_t eps_t phi~_t / sum_t phi~_t from the filtered densities
 * phi_tilde (device float[T][M], what update_field leaves in phi), the
 * generalised Poisson equation solved by the reference's polarisation
 * iteration (mixing, conv_crit, max_iter; conv_kind 0 max_diff, 1 csum,
 * 2 euclidean_norm as the mesh library's cnorm, a sum of squares),
 * psi = eps0^-1 (q + pol) / k^2 with q = rho~/eps, E = -grad psi,
 * V_t = q_t psi - (eps_t - eps) |E|^2 / (2 eps0^-1 sum phi~) and the forces
 * -grad(H * V_t) read out per type into elec_forces (device float[n][3]).
 * phi_eps and contrib (device float[M]) carry the reference's persistent
 * grids between calls (its masked divisions keep old values; zero them
 * before the first call).  pol_prev (device float[M]) is the starting
 * polarisation and is overwritten with the converged one; the reference
 * starts every solve from its caller's unchanged grid (field.py:1010-1024),
 * so the drop-in passes a copy.  Optional outputs (NULL to skip): psi,
 * elec_field (float[3][M]), elec_dot (|E|^2, float[M]), vbar (float[T][M]),
 * energy (device double: dV eps0/2 sum eps |E|^2).  The polarisation
 * iteration runs as a CUDA graph whose while node repeats the update while
 * the convergence test, evaluated on the device after each update, holds;
 * the graph is built on the first call and again when pol_prev, mixing,
 * conv_crit, conv_kind or max_iter change.  With iterations != NULL the call
 * synchronises the stream once, at its end, and *iterations receives their
 * number.  Not capturable: a stream under capture returns HPF_ERR_ARG. */
int hpf_gpe_step(hpf_ctx* ctx, const float* pos, const int32_t* types, const float* charges,
                 int64_t n, const float* phi_tilde, const double* eps_type,
                 const double* type_charges, double coulomb_constant, double conv_crit,
                 double mixing, int conv_kind, int max_iter, float* phi_eps, float* pol_prev,
                 float* contrib, float* elec_forces, float* psi, float* elec_field,
                 float* elec_dot, float* vbar, double* energy, int* iterations, void* stream);

/* ---- adjoint of the field energy ------------------------------------------
 * Gradients of W = sum_g w(phi~(g)) dV (hymd/field.py:688-703 with the
 * functional set by hpf_ctx_set_functional), for fitting the functional's
 * parameters; the reference has no gradient code (it uses the force, the
 * spectral readout of -grad V, which agrees with -dW/dx up to O(h^2)).
 * grad_pos (device float[n][3], or NULL): dW/dx, the exact derivative of the
 *   discrete W (CIC-weight gradient readout of H * Q phi~), FP32.
 * sums (device double[P + 1 + T], P = T(T+1)/2, or NULL): Parseval sums
 *   over the FP32 density spectra (FP32 products, compensated double-float
 *   reduction); with p_t = H phi_t(k) / M over the half spectrum:
 *   sums[p]   s_tj = sum_{k!=0} w_k Re(p_t conj p_j), p enumerating t <= j
 *             row-major, so sum_g phi~_t phi~_j dV = V (s_tj + mean_t mean_j);
 *   sums[P]   r = sum_{k!=0} w_k k^2 sum_tj Q_tj Re(p_t conj p_j), so that
 *             dW/dsigma = -sigma V r;
 *   sums[P+1+t] mean of phi_t.
 * Both parts share one paint and one r2c.  T <= 8 for sums
 * (HPF_ERR_NOT_IMPLEMENTED above). */
int hpf_field_adjoint(hpf_ctx* ctx, const float* pos, const int32_t* types, int64_t n,
                      const double* type_mass, float* grad_pos, double* sums, void* stream);

/* comp_laplacian (hymd/field.py:406-425): lap_out[t][d] = c2r(-k_d^2
 * phi_fourier[t]) for all T types and d = 0..2.  lap_out: float[T][3][M]. */
int hpf_laplacian(hpf_ctx* ctx, const void* phi_fourier, float* lap_out, void* stream);

/* ---- mesh -> particle ----------------------------------------------------
 * force[types == t, d] = force_mesh[t][d].readout(r[types == t])
 * (hymd/field.py:197-200).  force_mesh: float[T][3][M]; force: float[N][3]. */
int hpf_readout(hpf_ctx* ctx, const float* force_mesh, const float* pos,
                const int32_t* types, int64_t n, float* force, void* stream);

/* ---- whole field evaluation ----------------------------------------------
 * update_field + compute_field_force (field.py:428-616, 152-200) without the
 * real-space intermediates: paint -> r2c -> fused k-space -> c2r(3T) ->
 * readout.  Scratch spectra/grids belong to the context.  sums as in
 * hpf_kspace_force (may be NULL). */
int hpf_field_step(hpf_ctx* ctx, float* pos, const int32_t* types, int64_t n,
                   const double* type_mass, float* force, double* sums,
                   const double* pos_scale, const HpfKick* kick, void* stream);
/* Diagnostic: hpf_field_step with CUDA events between its stages; writes the
 * stage times in microseconds to the HOST array us_out[5] = {paint (incl.
 * fixed-point finalise), r2c, k-space, c2r, readout}.  Synchronises; not for
 * use inside a graph. */
int hpf_field_step_profile(hpf_ctx* ctx, float* pos, const int32_t* types, int64_t n,
                           const double* type_mass, float* force, double* sums,
                           const double* pos_scale, const HpfKick* kick, void* stream,
                           float* us_out);
/* pos_scale (device double, may be NULL): when given, positions are first
 * rescaled in place, pos = float(*pos_scale) * pos -- the position update of
 * a barostat step (hymd/barostat_scr.py:128) fused into the paint.
 * kick (may be NULL): the outer half kick (and CSVR sums) fused into the
 * readout, see HpfKick. */

/* ---- PIC_Spectral electrostatics ------------------------------------------
 * update_field_force_q (hymd/field.py:241-403): paint q/dV -> r2c -> H ->
 * psi = 4 pi k_e/eps H rho / k^2 (k=0 -> 1) -> E_d = -i k_d psi -> c2r ->
 * F = q readout(E).  Writes elec_forces float[N][3]; when non-null also
 * phi_q float[M], psi float[M], elec_field float[3][M], psi_k float2[Mc] and
 * sums[0] = sum_k w_k Re(rho_k conj psi_k) (k=0 included), so that
 * W_elec = V/2 sums[0] - E_self (field.py:698-699).  elec_factor = k_e/eps. */
int hpf_pic_step(hpf_ctx* ctx, const float* pos, const float* charges, int64_t n,
                 double elec_factor, float* elec_forces, float* phi_q, float* psi,
                 float* elec_field, void* psi_k, double* sums, const HpfKick* kick,
                 void* stream);
/* The same PIC step with the charge paint over a compact list of beads (the
 * charged ones): idx int32[count] (device) holds bead indices in [0, n).
 * Only those beads are painted (the reference paints every bead,
 * field.py:356-369, where q = 0 beads add nothing).  Without a kick only the
 * listed rows of elec_forces are read out and written (the others keep their
 * values); with a kick every bead is visited, as in hpf_pic_step (zero force
 * where q = 0), so that the kick and the CSVR sums cover all beads.  No grids
 * are returned.  sums as for hpf_pic_step. */
int hpf_pic_step_list(hpf_ctx* ctx, const float* pos, const float* charges, const int32_t* idx,
                      int64_t count, int64_t n, double elec_factor, float* elec_forces,
                      double* sums, const HpfKick* kick, void* stream);
/* Density and charge field step of one outer MD step in one call: the same
 * results as hpf_field_step(ctx, pos, types, n, type_mass, force, sums,
 * pos_scale, NULL, stream) followed by hpf_pic_step_list(ctx, pos, charges,
 * idx, count, n, elec_factor, elec_forces, pic_sums, kick, stream) -- the
 * reference's update_field + compute_field_force and update_field_force_q
 * of one step (main.py:606-660) -- with the charge chain (paint, transforms,
 * Poisson map) run on a second stream of the context beside the density
 * chain, joined before the charge readout, which carries the kick.  With
 * charges NULL (count 0) only the density chain runs and its readout
 * carries the kick, as hpf_field_step.  painted nonzero: this step's
 * deposits (densities, and charges when given) are already in the
 * context's accumulators, made by hpf_respa_step_paint, and the paints are
 * skipped; with pos_scale as well, those deposits were made at the positions
 * before the isotropic barostat's r -> alpha r (in the box before its
 * update, which gives the same grid coordinates), and the density readout
 * scales the positions by (float)pos_scale[0] as it reads them and writes
 * them back (as hpf_scr_scale_positions would, without its launch).  On the
 * fused spectral path only (painted or the second stream); otherwise the
 * two calls run one after the other.
 * The first call with charges allocates the charge chain's scratch (about
 * 3 Mc complex and 4 M real values) and must not be under stream capture
 * (HPF_ERR_ARG). */
int hpf_field_pic_step(hpf_ctx* ctx, float* pos, const int32_t* types, int64_t n,
                       const double* type_mass, float* force, double* sums,
                       const double* pos_scale, const float* charges, const int32_t* idx,
                       int64_t count, double elec_factor, float* elec_forces, double* pic_sums,
                       const HpfKick* kick, int painted, void* stream);

/* ---- bonded (f2py calling form, hymd/force.py:8-23, main.py:509-550) ------
 * All three zero their force array first, as the Fortran does.  Indices are
 * int32, 0-based.  out: device workspace (HPF_OUT_DOUBLES); out[0..3] =
 * {energy, virial_x, virial_y, virial_z} (virial = bond_pr / angle_pr).  d_err: device int (may be NULL)
 * receives HPF_ERR_INDEX for out-of-range indices (the term is skipped).
 * box: DEVICE double[3] (e.g. the context box state), so that a captured
 * graph follows box changes made on the device. */
/* cbf, hymd/compute_bond_forces.f90:1-61 */
int hpf_bonds(float* f, const float* r, int64_t n, const double box[3], const int32_t* a,
              const int32_t* b, const float* r0, const float* k, int64_t nb, double* out,
              int* d_err, void* stream);
/* caf, hymd/compute_angle_forces.f90:1-93 */
int hpf_angles(float* f, const float* r, int64_t n, const double box[3], const int32_t* a,
               const int32_t* b, const int32_t* c, const float* t0, const float* k,
               int64_t na, double* out, int* d_err, void* stream);
/* cdf, hymd/compute_dihedral_forces.f90:1-137 (+ dipole_reconstruction.f90).
 * coeff: float[D][6][5]; dtype, last: int32[D]; dipoles float[D][4][3];
 * transfer float[D][6][3][3] (both zeroed, written when dipole_flag = 1).
 * out: device workspace (HPF_OUT_DOUBLES); out[0] = energy. */
int hpf_dihedrals(float* f, const float* r, int64_t n, float* dipoles, float* transfer,
                  const double box[3], const int32_t* a, const int32_t* b, const int32_t* c,
                  const int32_t* d, const float* coeff, const int32_t* dtype,
                  const int32_t* last, int64_t nd, int dipole_flag, double* out, int* d_err,
                  void* stream);
/* dipole_forces_redistribution, hymd/force.py:855-877: zeroes f_on_bead
 * (float[N][3]) and adds the transfer-matrix images of the dipole forces. */
int hpf_dipole_redistribute(float* f_on_bead, int64_t n, const float* f_dipoles,
                            const float* transfer, const int32_t* a, const int32_t* b,
                            const int32_t* c, const int32_t* d, const int32_t* dtype,
                            const int32_t* last, int64_t nd, void* stream);

/* ---- integrator (hymd/integrator.py:9-73, main.py:802-887) ---------------
 * v += 0.5 dt F_i / mass for each of the n_f force arrays in order (one f32
 * rounding per array, as repeated integrate_velocity calls do). */
int hpf_kick(float* v, const float* const* forces, int n_f, int64_t n, double mass,
             double dt, void* stream);
/* Inner rRESPA step pieces: v += 0.5 dt (fb+fa+fd)/mass [times `kicks`],
 * then r = r + dt v when drift != 0, wrapped as np.mod(r, box) when box is
 * non-NULL.  fb/fa/fd may be NULL; box is a DEVICE double[3]. */
int hpf_inner_kick_drift(float* r, float* v, const float* fb, const float* fa,
                         const float* fd, int64_t n, double mass, double dt, int kicks,
                         int drift, const double box[3], void* stream);
/* FP64 sum of x[0..n) (y == NULL) or of x[e]*y[e] into out[0] (device
 * workspace, HPF_OUT_DOUBLES).  Used for csum-style grid reductions
 * (hymd/field.py:693, 699; hymd/pressure.py:100-121). */
int hpf_sum_dot(const float* x, const float* y, int64_t n, double* out, void* stream);
/* ---- fused rRESPA inner loop (hymd/main.py:802-887) -----------------------
 * A plan groups the beads joined by bonded terms into blocks of whole
 * molecules (connected components of the terms) of at most max_block_beads
 * beads, held in shared memory by one CTA each; beads in no term are "free".
 * All topology arrays are HOST arrays in the packed form of prepare_bonds
 * (hymd/force.py:573-728): int32 indices, float32 parameters, coeff
 * float[D][6][5].  Returns HPF_ERR_NOT_IMPLEMENTED when one molecule exceeds
 * the shared-memory capacity of a CTA (about 6400 beads); callers then use
 * the per-term entry points above. */
typedef struct hpf_respa_plan hpf_respa_plan;
int hpf_respa_plan_create(hpf_respa_plan** out, int64_t n_beads, int64_t nb, const int32_t* bond_a,
                          const int32_t* bond_b, const float* bond_r0, const float* bond_k,
                          int64_t na, const int32_t* ang_a, const int32_t* ang_b,
                          const int32_t* ang_c, const float* ang_t0, const float* ang_k,
                          int64_t nd, const int32_t* dih_a, const int32_t* dih_b,
                          const int32_t* dih_c, const int32_t* dih_d, const float* dih_coeff,
                          const int32_t* dih_type, const int32_t* dih_last, int max_block_beads);
int hpf_respa_plan_destroy(hpf_respa_plan* plan);
/* The bead arrays were permuted (a re-sort by mesh cell between steps):
 * inv (device int32[n], n = the plan's bead count) maps each old bead index
 * to its new one.  The groups' bead lists are remapped in place; the list of
 * free beads (in no bonded term) is replaced by free_ids (device
 * int32[n_free], the free beads' new indices, ascending, so that the free
 * beads are read in memory order), or remapped in place when free_ids is
 * NULL.  Graphs captured with this plan stay valid.  No counterpart in the
 * reference (its beads move between MPI ranks in domain_decomposition,
 * field.py:1115-1194, which rebuilds the bonded lists instead).  d_err
 * (device int, may be NULL) receives HPF_ERR_INDEX for an index outside
 * [0, n).  Stream-ordered; does not synchronise. */
int hpf_respa_plan_permute(hpf_respa_plan* plan, const int32_t* inv, int64_t n,
                           const int32_t* free_ids, int64_t n_free, int* d_err, void* stream);
/* Beads in molecule groups and free beads of a plan (host). */
int hpf_respa_plan_counts(const hpf_respa_plan* plan, int64_t* n_bonded, int64_t* n_free);
int hpf_respa_plan_info(const hpf_respa_plan* plan, int* n_mol_blocks, int* n_free,
                        int* max_block_beads);
/* hpf_respa_step (the launch itself) is declared after the barostat
 * arguments below. */


/* csvr_thermostat (hymd/thermostat.py:111-219) for up to two coupling groups.
 * The groups are visited in order, as the reference does: with COM removal
 * (and more than one particle) a group's particles are rescaled about the
 * group's COM velocity; otherwise K is the whole system's current kinetic
 * energy and every particle is scaled.  state: device double[16] ([4g] A_g,
 * [4g+1..3] B_g, the composed transform v <- A_g v + B_g of group g's
 * particles; [8+g] accumulated thermostat work).  ws: workspace
 * (HPF_OUT_DOUBLES). */
int hpf_csvr(float* v, const int32_t* group, int64_t n, const float* const* kick_forces,
             int n_kick, double kick_dt, const HpfCsvrArgs* args, const double* randoms,
             int* counter, double* state, double* ws, int* d_err, void* stream);
/* kick_forces (n_kick arrays, may be 0): the second outer half kick
 * v += 0.5 kick_dt F/mass (hymd/main.py:1143-1169) applied in the same pass,
 * before the kinetic energy is taken. */
/* The scaling half of hpf_csvr: v = A_g v + B_g from state
 * (hymd/thermostat.py:210-217); remove_com is carried by the transform in
 * state and is not read. */
int hpf_csvr_scale(float* v, const int32_t* group, int64_t n, const double* state,
                   int remove_com, void* stream);
/* Stochastic cell rescaling (hymd/barostat_scr.py): args->mode 0 isotropic
 * (:34-132), 1 semi-isotropic with z normal (:133-284).  The pressure from
 * field_sums (device double[4] = A, B_xyz of the last field evaluation, see
 * hpf_kspace_force), bonded_out (device double[9] of hpf_respa_step) and the
 * kinetic energy of v; then the box (the context's device box state, kept in
 * float32 values as the reference does) and the positions are rescaled as
 * hpf_scr_scale_positions does.  state[12] = alpha (semi: alpha_L),
 * state[13] = P (semi: P_L, bar), state[14] = alpha_N, state[15] = P_N,
 * state[10] = surface tension (semi, bar nm). */
int hpf_scr_isotropic(hpf_ctx* ctx, float* r, const float* v, int64_t n,
                      const double* field_sums, const double* bonded_out,
                      const HpfScrArgs* args, const double* randoms, int* counter,
                      double* state, double* ws, int* d_err, void* stream);
/* Position update of an SCR step from `state` (above).  mode 0: every
 * coordinate times alpha (barostat_scr.py:128).  mode 1: the reference's
 * `positions[:][0:2] *= alpha_L; positions[:][2] *= alpha_N` (:249, :280),
 * which index rows: all coordinates of particles 0 and 1 times alpha_L and
 * of particle 2 times alpha_N, the others unchanged. */
int hpf_scr_scale_positions(float* r, int64_t n, const double* state, int mode, void* stream);

/* One launch of the fused rRESPA inner loop: the first outer half kick
 * v += 0.5 respa_inner dt F_s / mass for each slow force array (field, PIC,
 * dipole, in that order, main.py:802-827), then respa_inner x [v += 0.5 dt
 * F_b/mass; r = mod(r + dt v, box); F_b = bonded forces(r); v += 0.5 dt
 * F_b/mass] (main.py:830-887).  f_bonded (float[N][3]) carries the bonded
 * force between calls and must hold the bonded force of the current
 * positions on entry (zero for free beads).  dipoles/transfer (may both be
 * NULL) receive the CBT dipoles of the last inner step (dipole_flag = 1
 * there, main.py:863-866).  out (device double[10], may be NULL) = {E_bond,
 * bond_pr[3], E_angle, angle_pr[3], E_dihedral, sum v^2} after the loop.
 * box: DEVICE double[3].
 * With baro != NULL the grid's last block then runs the isotropic SCR step
 * of hpf_scr_isotropic on the new box (field_sums, randoms, counter, state
 * as there; needs out); the positions are NOT rescaled here -- pass
 * &state[12] as pos_scale to the following hpf_field_step. */
int hpf_respa_step(hpf_respa_plan* plan, float* r, float* v, float* f_bonded,
                   const float* const* slow_forces, int n_slow, double mass, double dt,
                   int respa_inner, const double* box, float* dipoles, float* transfer,
                   double* out, hpf_ctx* baro_ctx, const HpfScrArgs* baro,
                   const double* field_sums, const double* randoms, int* counter, double* state,
                   int* d_err, void* stream);
/* hpf_respa_step with the paint of the next field step fused in: every
 * bead is deposited on field_ctx's accumulators where the kernel leaves its
 * final position -- a free bead right after its drift, while the molecule
 * groups still integrate; a group bead at the group's write-back -- into
 * its type's density grid and, when charges is non-NULL, into the charge
 * grid, the deposits of hpf_paint / hpf_pic_step (int64 fixed point, so
 * without a barostat the accumulators are bit-identical to a separate
 * paint).  The field step then runs with painted = 1 (hpf_field_pic_step).
 * baro (NULL: none) must be isotropic (mode 0; HPF_ERR_ARG otherwise): the
 * beads are deposited unscaled into the old box, which gives the grid
 * coordinates of the scaled positions in the new box (r n / L is unchanged
 * by r -> alpha r, L -> alpha L; equal up to FP32 rounding), and the caller
 * scales the positions afterwards (hpf_scr_scale_positions mode 0) and
 * runs the field step without pos_scale.  field_sums, randoms, counter and
 * state as for hpf_respa_step's barostat.  No counterpart in the
 * reference, where update_field paints after the inner loop and the
 * barostat (main.py:606-616, 889-963).  types int32[n] and charges float[n]
 * are device arrays of the plan's beads; d_err receives a non-finite
 * position or a type outside [0, T). */
int hpf_respa_step_paint(hpf_respa_plan* plan, float* r, float* v, float* f_bonded,
                         const float* const* slow_forces, int n_slow, double mass, double dt,
                         int respa_inner, const double* box, float* dipoles, float* transfer,
                         double* out, hpf_ctx* field_ctx, const int32_t* types,
                         const float* charges, const HpfScrArgs* baro, const double* field_sums,
                         const double* randoms, int* counter, double* state, int* d_err,
                         void* stream);

/* Bonded forces (bonds, angles, dihedrals with CBT) of the plan's topology at
 * positions r, without any integration: f_bonded of every bead in a bonded
 * term is overwritten with its force (other beads untouched), summed in the
 * plan's fixed incidence order, so the result is bit-reproducible (the
 * per-term kernels above accumulate with atomics).  out (device double[10]
 * or NULL): energies and virials as hpf_respa_step's out[0..8]; out[9] = 0.
 * The forces of compute_bond/angle/dihedral_forces (main.py:494-550) for the
 * first step of an rRESPA run. */
int hpf_respa_forces(hpf_respa_plan* plan, const float* r, float* f_bonded, const double* box,
                     double* out, int* d_err, void* stream);

/* Sum over particles of v^2 into out[0] (device workspace, HPF_OUT_DOUBLES);
 * KE = mass/2 * out[0]. */
int hpf_sum_v2(const float* v, int64_t n, double* out, void* stream);

/* ---- paint without allocation --------------------------------------------
 * No counterpart in the reference: a variant of hpf_paint (same densities,
 * bit for bit) for callers that hold no hpf_ctx and may not allocate device
 * memory.  Its scratch is one static device array per device of 16 MiB:
 * T * n0 * n1 * n2 <= 2^21 cells, beyond which it returns
 * HPF_ERR_SCRATCH_LIMIT.  It clears the accumulators itself on every call.
 * All calls on a device share that scratch, so calls that overlap in time (two
 * streams, two host threads) race; the first call on a device looks up the
 * array's address and should come before any stream capture (a first call
 * under capture returns HPF_ERR_ARG).  Each call outside a capture looks
 * the address up again, so after cudaDeviceReset one call outside a capture
 * makes later captured calls use the new context's array.  phi_out may
 * start at any 4-byte boundary.
 * box: host double[3]; type_mass: host double[T]; phi_out: float[T][M];
 * d_err: device int (may be NULL).                                         */
int hpf_paint_static(const float* pos, const int32_t* types, int64_t n, int T, int n0, int n1,
                     int n2, const double box[3], const double* type_mass, float* phi_out,
                     int* d_err, void* stream);

/* ---- topology preparation (hymd/force.py:325-505, prepare_bonds_old) ------
 * Finds the bonds, angles and dihedrals of every molecule from the bond rows
 * and the configured term types, in the order the reference's traversals
 * produce them (node insertion order; breadth-first depth 1 / 2 for bonds /
 * angles with gid(end) > gid(start); depth-first 4-node paths for
 * dihedrals, skipping a path whose reversed term is listed already), one
 * device thread per molecule.  All arrays are DEVICE arrays:
 *   mol_start  int[n_mol+1]  slot ranges of the molecules (ascending id);
 *   slot_bead  int[n_beads]  local bead at each slot (ascending within a
 *                            molecule, the reference's enumerate order);
 *   bead_slot  int[n_beads]  its inverse;
 *   gid        int64[n_beads] global index of each local bead (node key);
 *   name_id    int[n_beads]  small integer per distinct name;
 *   partners   int[n_beads][max_partners] bonded partners as LOCAL bead
 *                            indices, -1 for none (the bonds rows mapped
 *                            from global indices by the caller);
 *   bond_types int[nbt][2], angle_types int[nat][3], dih_types int[ndt][4]:
 *                            name ids of each configured type (-1 for a
 *                            name no bead has); dih_class: equal for types
 *                            with equal coefficients and dihedral type (the
 *                            reference's duplicate test compares those);
 *                            dih_bb: 1 where the dihedral type is 1;
 *   scratch    int[hpf_topology_scratch_ints(n_beads)].
 * offsets == NULL: counting pass, counts[n_mol][3] = (bonds, angles,
 * dihedrals) per molecule.  Otherwise the writing pass: offsets[n_mol][3]
 * (exclusive prefix sums of counts) place each molecule's terms in
 * bonds[B][3] = (i, j, type), angles[A][4] = (i, mid, j, type),
 * dihedrals[D][5] = (a, b, c, d, type) as local bead indices and indices into
 * the type arrays, and bb[n_mol] = index of the molecule's last type-1
 * dihedral or -1 (force.py:501-502).  d_err receives HPF_ERR_INDEX for a
 * partner outside its molecule and HPF_ERR_NOT_IMPLEMENTED for a node with
 * more than HPF_TOPO_MAX_DEGREE distinct neighbours. */
#define HPF_TOPO_MAX_DEGREE 8
int64_t hpf_topology_scratch_ints(int64_t n_beads);
int hpf_topology_terms(int64_t n_beads, int n_mol, const int* mol_start, const int* slot_bead,
                       const int* bead_slot, const long long* gid, const int* name_id,
                       const int* partners, int max_partners, const int* bond_types, int n_bond_types,
                       const int* angle_types, int n_angle_types, const int* dih_types,
                       const int* dih_class, const int* dih_bb, int n_dih_types, int* scratch,
                       int* counts, const int* offsets, int* bonds, int* angles, int* dihedrals,
                       int* bb, int* d_err, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* HPF_GB300_H */

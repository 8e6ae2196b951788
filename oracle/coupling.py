"""FP64 restatement of HyMD's temperature and pressure coupling (test
infrastructure only).

  csvr             hymd/thermostat.py:111-219 (canonical sampling through
                   velocity rescaling, Bussi-Parrinello 2008 form)
  scr_isotropic    hymd/barostat_scr.py:34-132 (stochastic cell rescaling)
  scr_semiisotropic hymd/barostat_scr.py:133-284 (z normal)

The random numbers come in as arguments, in the reference's draw order: per
coupling group one Gaussian then one chi^2_{N_f - 1}; per barostat step one
normal (semi-isotropic: lateral, then normal).
"""
import numpy as np

GAS_CONSTANT = 0.0083144621  # kJ mol^-1 K^-1, hymd/input_parser.py:159
BAR_PER_KJ_MOL_NM3 = 16.61  # the reference's pressure conversion, barostat_scr.py:98
BETA_WATER = 7.6e-4  # isothermal compressibility (1/bar), barostat_scr.py:77


def csvr(velocity, group, n_groups, mass, target_temperature, dt_outer, tau, draws,
         remove_com=True, gas_constant=GAS_CONSTANT):
    """thermostat.py:167-219.  `group` holds each particle's coupling group
    (0..n_groups-1), `draws` the (R, chi^2) pairs of the groups in order.
    The groups are visited in order and each visit acts on the velocities the
    previous one left: with COM removal (and more than one particle) the
    group's kinetic energy about its own COM velocity, and only the group's
    particles are rescaled about it; otherwise the whole system's kinetic
    energy, and every particle is scaled.  Returns (velocity, work)."""
    v = np.array(velocity, dtype=np.float64, copy=True)
    group = np.asarray(group)
    c = np.exp(-dt_outer / tau)
    work = 0.0
    for g in range(n_groups):
        sel = group == g
        n_g = int(np.sum(sel))
        use_com = remove_com and n_g > 1
        if use_com:
            com = v[sel].sum(axis=0) / n_g
            K = 0.5 * mass * np.sum((v[sel] - com) ** 2)
        else:
            K = 0.5 * mass * np.sum(v ** 2)
        K_target = 1.5 * gas_constant * n_g * target_temperature
        N_f = 3 * n_g
        R, S = draws[2 * g], draws[2 * g + 1]
        alpha2 = (c + (1 - c) * (S + R * R) * K_target / (N_f * K)
                  + 2 * R * np.sqrt(c * (1 - c) * K_target / (N_f * K)))
        work += K * (alpha2 - 1)
        alpha = np.sqrt(alpha2)
        if use_com:
            v[sel] = (v[sel] - com) * alpha + com
        else:
            v *= alpha
    return v, work


def _common_factor(n_b, dt_outer, tau_p, temperature, volume, gas_constant):
    return n_b * gas_constant * temperature * BETA_WATER * dt_outer * n_b / (volume * tau_p)


def scr_isotropic(pressure18, box, positions, R, target_pressure, tau_p, n_b, dt_outer,
                  temperature, gas_constant=GAS_CONSTANT):
    """barostat_scr.py:91-131: P = mean of the x and y total pressures (the
    reference's pressure[-3:-1]) in bar; log alpha' = -n_b dt beta / tau_p
    (P_target - P) + sqrt(2 ...) R; alpha = exp(log alpha' / 3); box and
    positions scaled by alpha.  Returns (box, positions, alpha)."""
    P = np.average(np.asarray(pressure18)[-3:-1]) * BAR_PER_KJ_MOL_NM3
    box = np.asarray(box, np.float64)
    V = float(np.prod(box))
    noise = np.sqrt(2.0 * _common_factor(n_b, dt_outer, tau_p, temperature, V, gas_constant)) * R
    log_alpha = -n_b * dt_outer * BETA_WATER / tau_p * (target_pressure - P) + noise
    alpha = np.exp(log_alpha / 3.0)
    return box * alpha, np.asarray(positions, np.float64) * alpha, alpha


def scr_semiisotropic(pressure18, box, positions, Rxy, Rz, target_l, target_n, tau_p, n_b,
                      dt_outer, temperature, gas_constant=GAS_CONSTANT):
    """barostat_scr.py:184-282 with z normal.  P_L = mean of the x and y total
    pressures, P_N the z one (bar); surface tension gamma = L_z/2 (P_N - P_L);
    a direction is coupled when its target is truthy.  The lateral step uses
    the volume before it, the normal step the volume after the lateral
    rescale.  The reference's position updates index rows, not columns
    (positions[:][0:2] and positions[:][2]): all coordinates of particles 0
    and 1 are scaled by alpha_L and those of particle 2 by alpha_N, and no
    other particle moves.  Returns (box, positions, alpha_L, alpha_N, gamma)."""
    p = np.asarray(pressure18)
    PL = (p[-3] + p[-2]) / 2 * BAR_PER_KJ_MOL_NM3
    PN = p[-1] * BAR_PER_KJ_MOL_NM3
    box = np.array(box, np.float64, copy=True)
    pos = np.array(positions, np.float64, copy=True)
    gamma = box[2] / 2 * (PN - PL)
    aL = aN = 1.0
    if target_l:
        V = float(np.prod(box))
        noise = np.sqrt(4.0 * _common_factor(n_b, dt_outer, tau_p, temperature, V, gas_constant)
                        / 3.0) * Rxy
        la = (-2.0 * n_b * dt_outer * BETA_WATER / (3 * tau_p)
              * (target_l - PL - gamma / box[2]) + noise)
        aL = np.exp(la / 2.0)
        box[0:2] *= aL
        pos[0:2] *= aL
    if target_n:
        V = float(np.prod(box))
        noise = np.sqrt(2.0 * _common_factor(n_b, dt_outer, tau_p, temperature, V, gas_constant)
                        / 3.0) * Rz
        la = -n_b * dt_outer * BETA_WATER / (3 * tau_p) * (target_n - PN) + noise
        aN = np.exp(la)
        box[2] *= aN
        pos[2] *= aN
    return box, pos, aL, aN, gamma

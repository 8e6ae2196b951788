/*
 * CPU oracle (test infrastructure only) -- body of the bonded-force restatement.
 *
 * Included twice by bonded_oracle.c: once with RT=float (the single-precision
 * f2py kernels cbf/caf/cdf) and once with RT=double (cbf_d/caf_d/cdf_d).
 * Arithmetic is real(8) throughout, as in the Fortran; values that the Fortran
 * stores in real(4) variables are rounded through RT at exactly those points.
 *
 * Reference files followed (paths inside the HyMD project):
 *   hymd/compute_bond_forces.f90:1-61        (cbf)
 *   hymd/compute_angle_forces.f90:1-93       (caf)
 *   hymd/compute_dihedral_forces.f90:1-137   (cdf)
 *   hymd/dipole_reconstruction.f90:1-221     (cross, cosine_series, reconstruct)
 * Arrays are C row-major: f, r (N,3); dipoles (D,4,3); transfer (D,6,3,3);
 * coeff (D,6,5) float32 (the Fortran declares coeff real(4) in both variants).
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)
#define RND(x) ((double)(RT)(x))

/* Fortran nint: round half away from zero. */
static double FN(orc_nint)(double x) { return round(x); }

static void FN(orc_min_image)(double v[3], const double box[3]) {
    for (int d = 0; d < 3; ++d) v[d] = v[d] - box[d] * FN(orc_nint)(v[d] / box[d]);
}

/* Difference of two stored positions: the Fortran subtracts in the storage
 * precision (real(4) for cbf/caf/cdf) and then widens. */
static void FN(orc_diff)(double out[3], const RT* r, int64_t i, int64_t j) {
    for (int d = 0; d < 3; ++d) out[d] = (double)(RT)(r[3 * i + d] - r[3 * j + d]);
}

static void FN(orc_cross)(double o[3], const double a[3], const double b[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

static double FN(orc_dot)(const double a[3], const double b[3]) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

static double FN(orc_norm2)(const double a[3]) { return sqrt(FN(orc_dot)(a, a)); }

/* force(i,:) = force(i,:) + s*v, rounded to storage precision */
static void FN(orc_acc)(RT* f, int64_t i, const double v[3], double s) {
    for (int d = 0; d < 3; ++d) f[3 * i + d] = (RT)((double)f[3 * i + d] + s * v[d]);
}

/* compute_bond_forces.f90:1-61 */
void FN(orc_bonds)(RT* f, const RT* r, int64_t n, const double* box,
                   const int64_t* a, const int64_t* b, const double* r0,
                   const double* k, int64_t nb, double* energy, RT* bond_pr) {
    *energy = 0.0;
    memset(f, 0, sizeof(RT) * 3 * n);
    /* bond_pr is intent(out) but never cleared by cbf; the oracle clears it. */
    bond_pr[0] = bond_pr[1] = bond_pr[2] = 0;
    for (int64_t ind = 0; ind < nb; ++ind) {
        int64_t aa = a[ind], bb = b[ind];
        double rab[3], fa[3];
        FN(orc_diff)(rab, r, bb, aa);
        FN(orc_min_image)(rab, box);
        double rn = FN(orc_norm2)(rab);
        double df = k[ind] * (rn - r0[ind]);
        for (int d = 0; d < 3; ++d) fa[d] = -df * rab[d] / rn;
        FN(orc_acc)(f, aa, fa, -1.0);
        FN(orc_acc)(f, bb, fa, 1.0);
        *energy = *energy + 0.5 * k[ind] * (rn - r0[ind]) * (rn - r0[ind]);
        for (int d = 0; d < 3; ++d) bond_pr[d] = (RT)((double)bond_pr[d] + fa[d] * rab[d]);
    }
}

/* compute_angle_forces.f90:1-93 */
void FN(orc_angles)(RT* f, const RT* r, int64_t n, const double* box,
                    const int64_t* a, const int64_t* b, const int64_t* c,
                    const double* t0, const double* k, int64_t na,
                    double* energy, RT* angle_pr) {
    *energy = 0.0;
    angle_pr[0] = angle_pr[1] = angle_pr[2] = 0;
    memset(f, 0, sizeof(RT) * 3 * n);
    for (int64_t ind = 0; ind < na; ++ind) {
        int64_t aa = a[ind], bb = b[ind], cc = c[ind];
        double ra[3], rc[3], ea[3], ec[3], fa[3], fc[3];
        FN(orc_diff)(ra, r, aa, bb);
        FN(orc_diff)(rc, r, cc, bb);
        FN(orc_min_image)(ra, box);
        FN(orc_min_image)(rc, box);
        double na_ = FN(orc_norm2)(ra), nc_ = FN(orc_norm2)(rc);
        for (int d = 0; d < 3; ++d) { ea[d] = ra[d] / na_; ec[d] = rc[d] / nc_; }
        double cosphi = FN(orc_dot)(ea, ec);
        double cosphi2 = cosphi * cosphi;
        if (cosphi2 < 1.0) {
            double theta = acos(cosphi);
            double sinphi = sin(theta);
            double dd = theta - t0[ind];
            double ff = k[ind] * dd;
            double xrasin = -ff / (na_ * sinphi);
            double xrcsin = -ff / (nc_ * sinphi);
            for (int d = 0; d < 3; ++d) {
                fa[d] = (ec[d] - cosphi * ea[d]) * xrasin;
                fc[d] = (ea[d] - cosphi * ec[d]) * xrcsin;
            }
            FN(orc_acc)(f, aa, fa, -1.0);
            FN(orc_acc)(f, cc, fc, -1.0);
            double s[3] = {fa[0] + fc[0], fa[1] + fc[1], fa[2] + fc[2]};
            FN(orc_acc)(f, bb, s, 1.0);
            *energy = *energy + 0.5 * ff * dd;
            for (int d = 0; d < 3; ++d)
                angle_pr[d] = (RT)((double)angle_pr[d] - (fa[d] * ra[d]) - (fc[d] * rc[d]));
        }
    }
}

/* dipole_reconstruction.f90:37-48 */
static void FN(orc_cosine_series)(const double* cn, const double* dn, double phi,
                                  double* e, double* de) {
    for (int i = 0; i < 5; ++i) {
        *e = *e + cn[i] * (1.0 + cos(i * phi - dn[i]));
        *de = *de - i * cn[i] * sin(i * phi - dn[i]);
    }
}

/* dipole_reconstruction.f90:50-220.  dipole: 2x3 RT block; tm: 3x3x3 RT block.
 * Where cos^2(gamma) >= 1 the Fortran leaves its intent(out) arguments
 * unassigned; the oracle defines them as zero. */
static void FN(orc_reconstruct)(const double rab[3], const RT* rb, const double rcb[3],
                                const double box[3], const double* c_k, const double* d_k,
                                double phi, int dipole_flag, double* e_cbt, double* df_cbt,
                                double fa[3], double fb[3], double fc[3], RT* dipole, RT* tm) {
    const double delta = 0.3;
    /* cos(1.392947) with a default-real literal: evaluated in real(4). */
    const double cos_psi = (double)(float)cos((double)1.392947f);
    const double sin_psi = (double)(float)sin((double)1.392947f);
    double k = 0.0, dk = 0.0;
    double gamma_0 = 1.85 - 0.227 * cos(phi - 0.785);
    double dg = 0.227 * sin(phi - 0.785);
    FN(orc_cosine_series)(c_k, d_k, phi, &k, &dk);
    double norm_a = FN(orc_norm2)(rab), norm_c = FN(orc_norm2)(rcb);
    double w[3], v[3];
    for (int d = 0; d < 3; ++d) { w[d] = rab[d] / norm_a; v[d] = rcb[d] / norm_c; }
    double cos_gamma = FN(orc_dot)(w, v);
    double cos2 = cos_gamma * cos_gamma;
    *e_cbt = 0.0; *df_cbt = 0.0;
    for (int d = 0; d < 3; ++d) fa[d] = fb[d] = fc[d] = 0.0;
    if (!(cos2 < 1.0)) return;
    double gamm = acos(cos_gamma);
    double sin_gamma = sqrt(1.0 - cos2);
    if (sin_gamma < (double)0.1f) sin_gamma = (double)0.1f; /* real(4) literal 0.1 */
    for (int d = 0; d < 3; ++d) {
        fa[d] = (v[d] - cos_gamma * w[d]) / norm_a;
        fc[d] = (w[d] - cos_gamma * v[d]) / norm_c;
        fa[d] = -fa[d] / sin_gamma;
        fc[d] = -fc[d] / sin_gamma;
        fb[d] = -(fa[d] + fc[d]);
    }
    double df_ang = k * (gamm - gamma_0);
    double var_sq = (gamm - gamma_0) * (gamm - gamma_0);
    *e_cbt = 0.5 * k * var_sq;
    *df_cbt = 0.5 * dk * var_sq - df_ang * dg;
    if (dipole_flag == 0) {
        for (int d = 0; d < 3; ++d) { fa[d] *= df_ang; fb[d] *= df_ang; fc[d] *= df_ang; }
        return;
    }
    double fac = exp((gamm - 1.73) / 0.025);
    double theta = -1.607 * gamm + 0.094 + 1.883 / (1.0 + fac);
    double d_theta = -1.607 - 1.883 / 0.025 * fac / ((1.0 + fac) * (1.0 + fac));
    double cos_theta = cos(theta), sin_theta = sin(theta);
    double nn[3], m[3], r0[3], dd[3], tmp[3];
    FN(orc_cross)(tmp, w, v);
    for (int d = 0; d < 3; ++d) nn[d] = tmp[d] / sin_gamma;
    FN(orc_cross)(m, nn, v);
    for (int d = 0; d < 3; ++d) {
        r0[d] = (double)rb[d] + 0.5 * rcb[d];
        dd[d] = 0.5 * delta * (cos_psi * v[d] + sin_psi * (cos_theta * nn[d] + sin_theta * m[d]));
    }
    for (int d = 0; d < 3; ++d) {
        dipole[0 * 3 + d] = (RT)(r0[d] + dd[d]);
        dipole[1 * 3 + d] = (RT)(r0[d] - dd[d]);
    }
    for (int p = 0; p < 2; ++p)
        for (int d = 0; d < 3; ++d) {
            double x = (double)dipole[p * 3 + d];
            dipole[p * 3 + d] = (RT)(x - box[d] * FN(orc_nint)(x / box[d]));
        }
    double Vb[3][3], Wb[3][3], Vc[3][3], Wa[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            Vb[i][j] = v[i] * v[j] - (i == j ? 1.0 : 0.0);
            Wb[i][j] = w[i] * w[j] - (i == j ? 1.0 : 0.0);
            Vb[i][j] /= norm_c;
            Wb[i][j] /= norm_a;
            Vc[i][j] = -Vb[i][j];
            Wa[i][j] = -Wb[i][j];
        }
    /* cross_matrix(M, x): row i = cross(M(i,:), x) */
    double cWa_v[3][3], cWb_v[3][3], cVb_w[3][3], cVc_w[3][3], cVb_n[3][3], cVc_n[3][3];
    for (int i = 0; i < 3; ++i) {
        FN(orc_cross)(cWa_v[i], Wa[i], v);
        FN(orc_cross)(cWb_v[i], Wb[i], v);
        FN(orc_cross)(cVb_w[i], Vb[i], w);
        FN(orc_cross)(cVc_w[i], Vc[i], w);
        FN(orc_cross)(cVb_n[i], Vb[i], nn);
        FN(orc_cross)(cVc_n[i], Vc[i], nn);
    }
    double Na[3][3], Nb[3][3], Nc[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            Na[i][j] = (cos_gamma * fa[i] * nn[j] + cWa_v[i][j]) / sin_gamma;
            Nb[i][j] = (cos_gamma * fb[i] * nn[j] + cWb_v[i][j] - cVb_w[i][j]) / sin_gamma;
            Nc[i][j] = (cos_gamma * fc[i] * nn[j] - cVc_w[i][j]) / sin_gamma;
        }
    double Ma[3][3], Mb[3][3], Mc[3][3];
    for (int i = 0; i < 3; ++i) {
        double t1[3];
        FN(orc_cross)(Ma[i], Na[i], v);
        FN(orc_cross)(t1, Nb[i], v);
        for (int j = 0; j < 3; ++j) Mb[i][j] = t1[j] - cVb_n[i][j];
        FN(orc_cross)(t1, Nc[i], v);
        for (int j = 0; j < 3; ++j) Mc[i][j] = t1[j] - cVc_n[i][j];
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double FNa = sin_theta * d_theta * fa[i] * nn[j];
            double FNb = sin_theta * d_theta * fb[i] * nn[j];
            double FNc = sin_theta * d_theta * fc[i] * nn[j];
            double FMa = cos_theta * d_theta * fa[i] * m[j];
            double FMb = cos_theta * d_theta * fb[i] * m[j];
            double FMc = cos_theta * d_theta * fc[i] * m[j];
            tm[0 * 9 + i * 3 + j] = (RT)(0.5 * delta * (sin_psi * (cos_theta * Na[i][j] + sin_theta * Ma[i][j] + FNa - FMa)));
            tm[1 * 9 + i * 3 + j] = (RT)(0.5 * delta * (cos_psi * Vb[i][j] + sin_psi * (cos_theta * Nb[i][j] + sin_theta * Mb[i][j] + FNb - FMb)));
            tm[2 * 9 + i * 3 + j] = (RT)(0.5 * delta * (cos_psi * Vc[i][j] + sin_psi * (cos_theta * Nc[i][j] + sin_theta * Mc[i][j] + FNc - FMc)));
        }
    for (int d = 0; d < 3; ++d) { fa[d] *= df_ang; fb[d] *= df_ang; fc[d] *= df_ang; }
}

/* compute_dihedral_forces.f90:1-137.  coeff is (D,6,5) float32 row-major. */
void FN(orc_dihedrals)(RT* force, const RT* r, int64_t n, RT* dipoles, RT* transfer,
                       const double* box, const int64_t* a, const int64_t* b,
                       const int64_t* c, const int64_t* d, const float* coeff,
                       const int64_t* dtype, const int64_t* last, int64_t nd,
                       int dipole_flag, double* energy) {
    *energy = 0.0;
    memset(force, 0, sizeof(RT) * 3 * n);
    memset(dipoles, 0, sizeof(RT) * 12 * nd);
    memset(transfer, 0, sizeof(RT) * 54 * nd);
    double phi = 0.0;
    for (int64_t ind = 0; ind < nd; ++ind) {
        int64_t aa = a[ind], bb = b[ind], cc = c[ind], dd = d[ind];
        double f[3], g[3], h[3], v[3], w[3], sc[3], fa[3], fb[3], fc[3], fd[3], mg[3];
        FN(orc_diff)(f, r, aa, bb);
        FN(orc_diff)(g, r, bb, cc);
        FN(orc_diff)(h, r, dd, cc);
        FN(orc_min_image)(f, box);
        FN(orc_min_image)(g, box);
        FN(orc_min_image)(h, box);
        FN(orc_cross)(v, f, g);
        FN(orc_cross)(w, h, g);
        double v_sq = FN(orc_dot)(v, v), w_sq = FN(orc_dot)(w, w);
        double g_norm = FN(orc_norm2)(g);
        double cos_phi = FN(orc_dot)(v, w);
        double sin_phi = FN(orc_dot)(w, f) * g_norm;
        /* The single-precision kernel keeps the previous phi when both vanish. */
        if (!(cos_phi == 0.0 && sin_phi == 0.0)) phi = atan2(sin_phi, cos_phi);
        double f_dot_g = FN(orc_dot)(f, g), h_dot_g = FN(orc_dot)(h, g);
        double df_dih = 0.0;
        const float* cf = coeff + 30 * ind;
        double row[6][5];
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 5; ++j) row[i][j] = (double)cf[i * 5 + j];
        if (dtype[ind] == 0 || dtype[ind] == 1) {
            df_dih = 0.0;
            FN(orc_cosine_series)(row[0], row[1], phi, energy, &df_dih);
            int nz_c = 0, nz_d = 0;
            for (int j = 0; j < 5; ++j) { nz_c += row[2][j] != 0.0; nz_d += row[3][j] != 0.0; }
            if (nz_c > 0 && nz_d > 0) FN(orc_cosine_series)(row[2], row[3], phi, energy, &df_dih);
        }
        if (dtype[ind] == 1) {
            double e_cbt, df_cbt;
            for (int q = 0; q < 3; ++q) mg[q] = -g[q];
            FN(orc_reconstruct)(f, r + 3 * bb, mg, box, row[4], row[5], phi, dipole_flag,
                                &e_cbt, &df_cbt, fa, fb, fc, dipoles + 12 * ind,
                                transfer + 54 * ind);
            *energy += e_cbt;
            df_dih += df_cbt;
            FN(orc_acc)(force, aa, fa, -1.0);
            FN(orc_acc)(force, bb, fb, -1.0);
            FN(orc_acc)(force, cc, fc, -1.0);
            if (last[ind] == 1) {
                FN(orc_reconstruct)(g, r + 3 * cc, h, box, row[4], row[5], phi, dipole_flag,
                                    &e_cbt, &df_cbt, fb, fc, fd, dipoles + 12 * ind + 6,
                                    transfer + 54 * ind + 27);
                *energy += e_cbt;
                df_dih += df_cbt;
                FN(orc_acc)(force, bb, fb, -1.0);
                FN(orc_acc)(force, cc, fc, -1.0);
                FN(orc_acc)(force, dd, fd, -1.0);
            }
        }
        if (dtype[ind] == 2) {
            double eq = row[0][0], kc = row[0][1];
            df_dih = kc * (phi - eq);
            *energy = *energy + 0.5 * kc * (phi - eq) * (phi - eq);
        }
        for (int q = 0; q < 3; ++q) {
            sc[q] = v[q] * f_dot_g / (v_sq * g_norm) - w[q] * h_dot_g / (w_sq * g_norm);
            fa[q] = -df_dih * g_norm * v[q] / v_sq;
            fd[q] = df_dih * g_norm * w[q] / w_sq;
            fb[q] = df_dih * sc[q] - fa[q];
            fc[q] = -df_dih * sc[q] - fd[q];
        }
        FN(orc_acc)(force, aa, fa, 1.0);
        FN(orc_acc)(force, bb, fb, 1.0);
        FN(orc_acc)(force, cc, fc, 1.0);
        FN(orc_acc)(force, dd, fd, 1.0);
    }
}

#undef FN
#undef RND

/*
 * Field loops of the CPU oracle -- TEST INFRASTRUCTURE ONLY (see oracle_common.h).
 *
 * Instantiated by axs_oracle.c once per precision with
 *   REAL = double, FN(x) = x##_f64   (the reference's PRECISION=DOUBLE build)
 *   REAL = float,  FN(x) = x##_f32   (the reference's default PRECISION=FLOAT
 *                                     build, AxionStrings/GNUmakefile:31)
 *
 * Layout: one AMReX FArrayBox -- component-major SoA, x fastest, every
 * direction padded by `ng` ghost cells (AxionStringsRHS.impl.hpp:29-36):
 *   idx(i,j,k,c) = (i+ng) + (j+ng)*js + (k+ng)*ks + c*cs,
 *   js = nx+2ng, ks = js*(ny+2ng), cs = ks*(nz+2ng).
 * The domain is one periodic box (the single-level uniform-grid case).
 */

typedef struct {
    int nx, ny, nz, ng;
    int64_t js, ks, cs;
} FN(orc_box);

static inline FN(orc_box) FN(orc_make_box)(int nx, int ny, int nz, int ng)
{
    FN(orc_box) b;
    b.nx = nx; b.ny = ny; b.nz = nz; b.ng = ng;
    b.js = nx + 2 * ng;
    b.ks = b.js * (ny + 2 * ng);
    b.cs = b.ks * (nz + 2 * ng);
    return b;
}

static inline int64_t FN(orc_idx)(const FN(orc_box) *b, int i, int j, int k)
{
    return (int64_t)(i + b->ng) + (int64_t)(j + b->ng) * b->js + (int64_t)(k + b->ng) * b->ks;
}

static inline int FN(orc_wrap)(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}

/* Periodic ghost fill of every component (AMReX FillBoundary(periodicity),
 * called before each RHS evaluation and each diagnostic,
 * AxionStringsLevel.cpp:1255). Fills edges and corners too. */
void FN(oracle_fill_periodic)(REAL *f, int nx, int ny, int nz, int ng, int ncomp)
{
    const FN(orc_box) b = FN(orc_make_box)(nx, ny, nz, ng);
    for (int c = 0; c < ncomp; ++c) {
        REAL *p = f + (int64_t)c * b.cs;
#pragma omp parallel for schedule(static)
        for (int k = -ng; k < nz + ng; ++k)
            for (int j = -ng; j < ny + ng; ++j)
                for (int i = -ng; i < nx + ng; ++i) {
                    if (i >= 0 && i < nx && j >= 0 && j < ny && k >= 0 && k < nz) continue;
                    p[FN(orc_idx)(&b, i, j, k)] =
                        p[FN(orc_idx)(&b, FN(orc_wrap)(i, nx), FN(orc_wrap)(j, ny), FN(orc_wrap)(k, nz))];
                }
    }
}

/* GRTeclyn FourthOrderDerivatives::diff2 / diff1 (third-party, absent from
 * the reference tree; called at AxionStringsRHS.impl.hpp:20 and through
 * d1_scalar at EnergyKernel.hpp:159-160). Restated from the published
 * GRChombo/GRTeclyn form: centred 5-point weights (1/12, 4/3, 5/2) and
 * (1/12, 2/3), evaluated in double, scaled by 1/dx^2 resp. 1/dx. */
static inline REAL FN(orc_diff2)(const REAL *in, int64_t s, double one_over_dx2)
{
    const double wf = 8.33333333333333333333e-2;
    const double wn = 1.33333333333333333333e+0;
    const double wl = 2.50000000000000000000e+0;
    return (REAL)((-wf * (double)in[-2 * s] + wn * (double)in[-s] - wl * (double)in[0] +
                   wn * (double)in[s] - wf * (double)in[2 * s]) *
                  one_over_dx2);
}

static inline REAL FN(orc_diff1)(const REAL *in, int64_t s, double one_over_dx)
{
    const double wf = 8.33333333333333333333e-2;
    const double wn = 6.66666666666666666667e-1;
    return (REAL)((wf * (double)in[-2 * s] - wn * (double)in[-s] + wn * (double)in[s] -
                   wf * (double)in[2 * s]) *
                  one_over_dx);
}

/* AxionStringsRHS<FourthOrderDerivatives>::operator()
 * (AxionStrings/AxionStringsRHS.impl.hpp:25-60) over the valid cells of one
 * box. `soln` must have >= 2 filled ghost layers. Coefficients are passed as
 * amrex::Real, as the reference's constructor takes them
 * (AxionStringsRHS.hpp:32-33). */
void FN(oracle_rhs)(const REAL *soln, REAL *rhs, int nx, int ny, int nz, int ng, double dx,
                    double kappa_d, double lambda_d, double R2_d)
{
    const FN(orc_box) b = FN(orc_make_box)(nx, ny, nz, ng);
    const REAL kappa = (REAL)kappa_d, lambda = (REAL)lambda_d, R2 = (REAL)R2_d;
    const double one_over_dx2 = 1.0 / (dx * dx);
    const int64_t strides[3] = {1, b.js, b.ks};
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int64_t o = FN(orc_idx)(&b, i, j, k);
                REAL lap1 = 0.0, lap2 = 0.0;
                for (int d = 0; d < 3; ++d) {
                    lap1 += FN(orc_diff2)(soln + 0 * b.cs + o, strides[d], one_over_dx2);
                }
                for (int d = 0; d < 3; ++d) {
                    lap2 += FN(orc_diff2)(soln + 1 * b.cs + o, strides[d], one_over_dx2);
                }
                const REAL psi1 = soln[0 * b.cs + o];
                const REAL psi2 = soln[1 * b.cs + o];
                const REAL d = psi1 * psi1 + psi2 * psi2 - R2;
                const REAL pc = (REAL)(0.5 * (double)lambda * (double)d);
                rhs[0 * b.cs + o] = soln[2 * b.cs + o];
                rhs[1 * b.cs + o] = soln[3 * b.cs + o];
                rhs[2 * b.cs + o] = lap1 + kappa * psi1 - pc * psi1;
                rhs[3 * b.cs + o] = lap2 + kappa * psi2 - pc * psi2;
            }
}

/* dst = x + a*y over the valid cells of all 4 components (AMReX
 * MultiFab::LinComb with unit first weight, as the RK stages use it). */
static void FN(orc_lincomb)(REAL *dst, const REAL *x, REAL a, const REAL *y, const FN(orc_box) *b)
{
    for (int c = 0; c < 4; ++c) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < b->nz; ++k)
            for (int j = 0; j < b->ny; ++j)
                for (int i = 0; i < b->nx; ++i) {
                    const int64_t o = c * b->cs + FN(orc_idx)(b, i, j, k);
                    dst[o] = x[o] + a * y[o];
                }
    }
}

/* Classic 4-stage Runge-Kutta on one periodic box, in the method-of-lines
 * form the reference delegates to GRTeclyn/AMReX (docs/conventions.md:239-245;
 * the RK driver itself is third-party and absent). Per stage: periodic ghost
 * fill, RHS at the stage time t, t+dt/2, t+dt/2, t+dt with the Background
 * coefficients at tau = tau_i + t_stage (AxionStringsLevel.cpp:878-907),
 * stage state U_s = U_old + c_s dt k_{s-1}; final U_old + dt/6 (k1+2k2+2k3+k4).
 * `state` has ng >= 2 ghosts; on return its ghosts are refilled. */
int FN(oracle_rk4_advance)(REAL *state, int nx, int ny, int nz, int ng, double dx,
                           const orc_background *bg, double tau_i, double t0, double dt,
                           int nsteps)
{
    if (ng < 2) return -1;
    const FN(orc_box) b = FN(orc_make_box)(nx, ny, nz, ng);
    const size_t n = (size_t)(4 * b.cs);
    REAL *uold = (REAL *)calloc(n, sizeof(REAL));
    REAL *ustage = (REAL *)calloc(n, sizeof(REAL));
    REAL *kk[4];
    for (int s = 0; s < 4; ++s) kk[s] = (REAL *)calloc(n, sizeof(REAL));
    if (!uold || !ustage || !kk[0] || !kk[1] || !kk[2] || !kk[3]) return -2;
    double t = t0;
    for (int step = 0; step < nsteps; ++step) {
        memcpy(uold, state, n * sizeof(REAL));
        const double ts[4] = {t, t + 0.5 * dt, t + 0.5 * dt, t + dt};
        const double cs[3] = {0.5 * dt, 0.5 * dt, dt};
        for (int s = 0; s < 4; ++s) {
            REAL *u = (s == 0) ? uold : ustage;
            FN(oracle_fill_periodic)(u, nx, ny, nz, ng, 4);
            double kap, lam, r2;
            orc_bg_rhs_coeffs(bg, tau_i + ts[s], &kap, &lam, &r2);
            FN(oracle_rhs)(u, kk[s], nx, ny, nz, ng, dx, kap, lam, r2);
            if (s < 3) FN(orc_lincomb)(ustage, uold, (REAL)cs[s], kk[s], &b);
        }
        const REAL h6 = (REAL)(dt / 6.0);
        for (int c = 0; c < 4; ++c) {
#pragma omp parallel for schedule(static)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        const int64_t o = c * b.cs + FN(orc_idx)(&b, i, j, k);
                        state[o] = uold[o] + h6 * (kk[0][o] + (REAL)2 * kk[1][o] +
                                                   (REAL)2 * kk[2][o] + kk[3][o]);
                    }
        }
        t = t0 + (step + 1) * dt;
    }
    FN(oracle_fill_periodic)(state, nx, ny, nz, ng, 4);
    free(uold); free(ustage);
    for (int s = 0; s < 4; ++s) free(kk[s]);
    return 0;
}

/* StringFinder.hpp:45-68 (plaquette_windings_at: 7 corner phases from
 * double atan2; xy, yz, zx loops at the low-index corner) and :76-122
 * (count_plaquettes: n_p_plain = # pierced, n_p_weighted = sum |w|, optional
 * coverage mask). `state` needs >= 1 filled ghost layer. `w_out` (nullable)
 * receives int8 windings [cell][plane], cell = i + nx*(j + ny*k). */
void FN(oracle_count_plaquettes)(const REAL *state, int nx, int ny, int nz, int ng,
                                 const uint8_t *mask, int64_t *n_plain, int64_t *n_weighted,
                                 int8_t *w_out)
{
    const FN(orc_box) b = FN(orc_make_box)(nx, ny, nz, ng);
    const REAL *p1 = state, *p2 = state + b.cs;
    int64_t plain = 0, weighted = 0;
#pragma omp parallel for schedule(static) reduction(+ : plain, weighted)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int64_t cell = i + (int64_t)nx * (j + (int64_t)ny * k);
                if (mask && mask[cell] == 0) {
                    if (w_out) w_out[3 * cell] = w_out[3 * cell + 1] = w_out[3 * cell + 2] = 0;
                    continue;
                }
#define ORC_PH(ii, jj, kk) \
    atan2((double)p2[FN(orc_idx)(&b, ii, jj, kk)], (double)p1[FN(orc_idx)(&b, ii, jj, kk)])
                const double th_000 = ORC_PH(i, j, k);
                const double th_100 = ORC_PH(i + 1, j, k);
                const double th_110 = ORC_PH(i + 1, j + 1, k);
                const double th_010 = ORC_PH(i, j + 1, k);
                const double th_001 = ORC_PH(i, j, k + 1);
                const double th_101 = ORC_PH(i + 1, j, k + 1);
                const double th_011 = ORC_PH(i, j + 1, k + 1);
#undef ORC_PH
                const int wxy = orc_plaquette_winding(th_000, th_100, th_110, th_010);
                const int wyz = orc_plaquette_winding(th_000, th_010, th_011, th_001);
                const int wzx = orc_plaquette_winding(th_000, th_001, th_101, th_100);
                plain += (wxy != 0) + (wyz != 0) + (wzx != 0);
                weighted += abs(wxy) + abs(wyz) + abs(wzx);
                if (w_out) {
                    w_out[3 * cell] = (int8_t)wxy;
                    w_out[3 * cell + 1] = (int8_t)wyz;
                    w_out[3 * cell + 2] = (int8_t)wzx;
                }
            }
    *n_plain = plain;
    *n_weighted = weighted;
}

/* AxionStringsLevel::apply_pre_evolution_to_main_rescale (AxionStringsLevel.cpp:2027-2132):
 * in place over every cell including ghosts; R's and kappa as amrex::Real. */
void FN(oracle_handoff_rescale)(REAL *state, int nx, int ny, int nz, int ng, double R_pre_d, double R_pre_prime_d,
                                double R_main_d, double R_main_prime_d)
{
    const FN(orc_box) b = FN(orc_make_box)(nx, ny, nz, ng);
    const REAL R_pre = (REAL)R_pre_d, R_pre_prime = (REAL)R_pre_prime_d;
    const REAL R_main = (REAL)R_main_d, R_main_prime = (REAL)R_main_prime_d;
    const REAL kappa = R_main / R_pre;
    const REAL common_term = R_main_prime - kappa * kappa * R_pre_prime;
    for (int64_t o = 0; o < b.cs; ++o) {
        const REAL psi1 = state[o], psi2 = state[b.cs + o], Pi1 = state[2 * b.cs + o], Pi2 = state[3 * b.cs + o];
        state[o] = kappa * psi1;
        state[b.cs + o] = kappa * psi2;
        state[2 * b.cs + o] = kappa * kappa * Pi1 + (psi1 / R_pre) * common_term;
        state[3 * b.cs + o] = kappa * kappa * Pi2 + (psi2 / R_pre) * common_term;
    }
}

/* fill_masked_a_dot_buffer (MaskedFieldBuffer.hpp:15-35): buf[cell] =
 * (REAL) masked_a_dot(psi1, psi2, Pi1, Pi2, R), R passed as amrex::Real. */
void FN(oracle_masked_a_dot_buffer)(const REAL *state, int nx, int ny, int nz, int ng, int scheme,
                                    double threshold, double R_d, REAL *buf)
{
    const FN(orc_box) b = FN(orc_make_box)(nx, ny, nz, ng);
    const double R = (double)(REAL)R_d;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int64_t o = FN(orc_idx)(&b, i, j, k);
                buf[i + (int64_t)nx * (j + (int64_t)ny * k)] = (REAL)orc_masked_a_dot(
                    scheme, threshold, state[o], state[b.cs + o], state[2 * b.cs + o], state[3 * b.cs + o], R);
            }
}

/* StringTagger::operator() (StringTagger.hpp:117-151): a cell is tagged when
 * a plaquette at its low corner is pierced (plaquette_windings_at, the string
 * finder's own test), or when dx^2 |lap psi_i| > gradient_threshold
 * (scalar_laplacian, :159-177: sum over d of diff2 as amrex::Real, summed in
 * double), or when dx |grad r| > radial_gradient_threshold (radial_gradient_sq,
 * :187-217). Then the n_error_buf buffer AMReX's TagBoxArray::buffer applies
 * before clustering: every cell within nbuf cells (a cube) of a tag is tagged,
 * wrapping periodically on this one-box periodic domain. tags[cell] = 1/0,
 * cell = i + nx*(j + ny*k). `state` needs >= 2 filled ghost layers. */
void FN(oracle_tag_cells)(const REAL *state, int nx, int ny, int nz, int ng, double dx_d, double grad_thr,
                          double rad_thr, int nbuf, uint8_t *tags)
{
    const FN(orc_box) b = FN(orc_make_box)(nx, ny, nz, ng);
    const int64_t n = (int64_t)nx * ny * nz;
    int8_t *w = (int8_t *)malloc((size_t)(3 * n));
    int64_t np, nw;
    FN(oracle_count_plaquettes)(state, nx, ny, nz, ng, NULL, &np, &nw, w);
    const REAL dx = (REAL)dx_d;
    const double dx2 = (double)(dx * dx);
    const double one_over_dx2 = 1.0 / (dx_d * dx_d), one_over_dx = 1.0 / dx_d;
    const int64_t strides[3] = {1, b.js, b.ks};
    uint8_t *t0 = (uint8_t *)malloc((size_t)n);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int64_t cell = i + (int64_t)nx * (j + (int64_t)ny * k);
                const int64_t o = FN(orc_idx)(&b, i, j, k);
                uint8_t tag = (w[3 * cell] | w[3 * cell + 1] | w[3 * cell + 2]) != 0;
                if (!tag) {
                    double lap1 = 0.0, lap2 = 0.0;
                    for (int d = 0; d < 3; ++d) {
                        lap1 += (double)FN(orc_diff2)(state + o, strides[d], one_over_dx2);
                        lap2 += (double)FN(orc_diff2)(state + b.cs + o, strides[d], one_over_dx2);
                    }
                    tag = dx2 * fabs(lap1) > grad_thr || dx2 * fabs(lap2) > grad_thr;
                }
                if (!tag) {
                    const double psi1 = state[o], psi2 = state[b.cs + o];
                    const double psi_sq = psi1 * psi1 + psi2 * psi2;
                    double g1 = 0.0, g2 = 0.0, gt = 0.0;
                    for (int d = 0; d < 3; ++d) {
                        const double d1 = (double)FN(orc_diff1)(state + o, strides[d], one_over_dx);
                        const double d2 = (double)FN(orc_diff1)(state + b.cs + o, strides[d], one_over_dx);
                        g1 += d1 * d1;
                        g2 += d2 * d2;
                        const double dth = psi_sq > 0.0 ? (psi1 * d2 - psi2 * d1) / psi_sq : 0.0;
                        gt += dth * dth;
                    }
                    tag = (double)dx * sqrt(g1 + g2 - psi_sq * gt) > rad_thr;
                }
                t0[cell] = tag;
            }
    free(w);
    if (nbuf <= 0) {
        memcpy(tags, t0, (size_t)n);
        free(t0);
        return;
    }
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                uint8_t any = 0;
                for (int dk = -nbuf; dk <= nbuf && !any; ++dk)
                    for (int dj = -nbuf; dj <= nbuf && !any; ++dj)
                        for (int di = -nbuf; di <= nbuf && !any; ++di) {
                            const int ii = FN(orc_wrap)(i + di, nx), jj = FN(orc_wrap)(j + dj, ny),
                                      kk = FN(orc_wrap)(k + dk, nz);
                            any = t0[ii + (int64_t)nx * (jj + (int64_t)ny * kk)];
                        }
                tags[i + (int64_t)nx * (j + (int64_t)ny * k)] = any;
            }
    free(t0);
}

/* EnergyKernel.hpp:106-233 (compute_total_energy_sums): the 14 per-cell
 * sums {rho, rho w, a_kin, a_kin w, a_grad, a_grad w, r_kin, r_kin w,
 * r_grad, r_grad w, r_mass, r_mass w, w, 1} in that order, 4th-order diff1
 * gradients, psi_sq > 0 guards. R, lambda, R'/R and dx enter as amrex::Real
 * (EnergyKernel.hpp:107-109). Accumulated with compensated summation so the
 * oracle's sums are accurate to ~1 ulp. `state` needs >= 2 ghost layers. */
void FN(oracle_energy_sums)(const REAL *state, int nx, int ny, int nz, int ng, double dx_d,
                            double R_d, double lambda_d, double RpR_d, int scheme,
                            double threshold, const uint8_t *mask, double out[14])
{
    const FN(orc_box) b = FN(orc_make_box)(nx, ny, nz, ng);
    const REAL dx = (REAL)dx_d;
    const double R = (REAL)R_d, lambda = (REAL)lambda_d, RpR = (REAL)RpR_d;
    const double one_over_dx = 1.0 / (double)dx;
    const int64_t strides[3] = {1, b.js, b.ks};
    orc_ksum tot[14];
    memset(tot, 0, sizeof(tot));
#pragma omp parallel
    {
        orc_ksum acc[14];
        memset(acc, 0, sizeof(acc));
#pragma omp for schedule(static)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const int64_t cell = i + (int64_t)nx * (j + (int64_t)ny * k);
                    if (mask && mask[cell] == 0) continue;
                    const int64_t o = FN(orc_idx)(&b, i, j, k);
                    const double psi1 = state[o], psi2 = state[b.cs + o];
                    const double Pi1 = state[2 * b.cs + o], Pi2 = state[3 * b.cs + o];
                    const double psi_sq = psi1 * psi1 + psi2 * psi2;
                    double g1sq = 0.0, g2sq = 0.0, gtsq = 0.0;
                    for (int d = 0; d < 3; ++d) {
                        const REAL g1 = FN(orc_diff1)(state + o, strides[d], one_over_dx);
                        const REAL g2 = FN(orc_diff1)(state + b.cs + o, strides[d], one_over_dx);
                        g1sq += g1 * g1;
                        g2sq += g2 * g2;
                        const double dth = (psi_sq > 0.0) ? (psi1 * g2 - psi2 * g1) / psi_sq : 0.0;
                        gtsq += dth * dth;
                    }
                    const double rho = orc_rho_tot(psi1, psi2, Pi1, Pi2, g1sq, g2sq, R, lambda, RpR);
                    const double thp = (psi_sq > 0.0) ? (psi1 * Pi2 - Pi1 * psi2) / psi_sq : 0.0;
                    const double akin = orc_axion_kinetic(thp, R);
                    const double agrad = orc_axion_gradient(gtsq, R);
                    const double rkin = orc_radial_kinetic(psi1, psi2, Pi1, Pi2, R, RpR);
                    const double rgrad = orc_radial_gradient(g1sq, g2sq, psi_sq, gtsq, R);
                    const double rmass = orc_radial_mass(psi1, psi2, R, lambda);
                    const double w = orc_masking_weight(scheme, threshold, psi1, psi2, R);
                    const double v[14] = {rho,   rho * w,   akin,  akin * w,  agrad,
                                          agrad * w, rkin, rkin * w, rgrad, rgrad * w,
                                          rmass, rmass * w, w,     1.0};
                    for (int q = 0; q < 14; ++q) orc_kadd(&acc[q], v[q]);
                }
#pragma omp critical
        for (int q = 0; q < 14; ++q) {
            orc_kadd(&tot[q], acc[q].s);
            orc_kadd(&tot[q], acc[q].c);
        }
    }
    for (int q = 0; q < 14; ++q) out[q] = orc_kval(&tot[q]);
}

/* VelocityKernel.hpp:37-141 (compute_velocity_at_pierced_corners): the three
 * windings recomputed with atan2 on amrex::Real (float atan2 in a FLOAT
 * build, VelocityKernel.hpp:66-69), gamma^2 v^2 (Velocity.hpp:62-78) summed
 * over the 4 corners of each pierced plaquette, count += 4 per plaquette. */
void FN(oracle_velocity)(const REAL *state, int nx, int ny, int nz, int ng, double R_d,
                         double RpR_d, double m_r_d, const uint8_t *mask, double *sum_out,
                         int64_t *count_out)
{
    const FN(orc_box) b = FN(orc_make_box)(nx, ny, nz, ng);
    const double R = (REAL)R_d, inv_bt = (REAL)RpR_d, m_r = (REAL)m_r_d;
    const REAL *p1 = state, *p2 = state + b.cs, *q1 = state + 2 * b.cs, *q2 = state + 3 * b.cs;
    orc_ksum tot = {0, 0};
    int64_t count = 0;
#pragma omp parallel reduction(+ : count)
    {
        orc_ksum acc = {0, 0};
#pragma omp for schedule(static)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const int64_t cell = i + (int64_t)nx * (j + (int64_t)ny * k);
                    if (mask && mask[cell] == 0) continue;
#define ORC_PH(ii, jj, kk) \
    ((double)FN(orc_atan2)(p2[FN(orc_idx)(&b, ii, jj, kk)], p1[FN(orc_idx)(&b, ii, jj, kk)]))
#define ORC_GVV(ii, jj, kk)                                                                   \
    orc_gamma_sq_v_sq_from_phi(                                                                \
        (double)p1[FN(orc_idx)(&b, ii, jj, kk)] / R, (double)p2[FN(orc_idx)(&b, ii, jj, kk)] / R, \
        ((double)q1[FN(orc_idx)(&b, ii, jj, kk)] - inv_bt * (double)p1[FN(orc_idx)(&b, ii, jj, kk)]) / (R * R), \
        ((double)q2[FN(orc_idx)(&b, ii, jj, kk)] - inv_bt * (double)p2[FN(orc_idx)(&b, ii, jj, kk)]) / (R * R), \
        m_r)
                    const double th_000 = ORC_PH(i, j, k);
                    const double th_100 = ORC_PH(i + 1, j, k);
                    const double th_110 = ORC_PH(i + 1, j + 1, k);
                    const double th_010 = ORC_PH(i, j + 1, k);
                    const double th_001 = ORC_PH(i, j, k + 1);
                    const double th_101 = ORC_PH(i + 1, j, k + 1);
                    const double th_011 = ORC_PH(i, j + 1, k + 1);
                    const int wxy = orc_plaquette_winding(th_000, th_100, th_110, th_010);
                    const int wyz = orc_plaquette_winding(th_000, th_010, th_011, th_001);
                    const int wzx = orc_plaquette_winding(th_000, th_001, th_101, th_100);
                    double s = 0.0;
                    int64_t c = 0;
                    if (wxy != 0) {
                        s += ORC_GVV(i, j, k) + ORC_GVV(i + 1, j, k) + ORC_GVV(i + 1, j + 1, k) +
                             ORC_GVV(i, j + 1, k);
                        c += 4;
                    }
                    if (wyz != 0) {
                        s += ORC_GVV(i, j, k) + ORC_GVV(i, j + 1, k) + ORC_GVV(i, j + 1, k + 1) +
                             ORC_GVV(i, j, k + 1);
                        c += 4;
                    }
                    if (wzx != 0) {
                        s += ORC_GVV(i, j, k) + ORC_GVV(i, j, k + 1) + ORC_GVV(i + 1, j, k + 1) +
                             ORC_GVV(i + 1, j, k);
                        c += 4;
                    }
#undef ORC_PH
#undef ORC_GVV
                    if (c) orc_kadd(&acc, s);
                    count += c;
                }
#pragma omp critical
        {
            orc_kadd(&tot, acc.s);
            orc_kadd(&tot, acc.c);
        }
    }
    *sum_out = orc_kval(&tot);
    *count_out = count;
}

/*
 * CPU oracle for the axion-string hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library (through oracle/oracle.py), as the checker and as the timed
 * CPU baseline. The GPU library never links or calls it.
 *
 * Build: oracle/Makefile (gcc -O3 -fopenmp -ffp-contract=off). Contraction is
 * off so x86_64 and aarch64 builds evaluate the same expressions.
 */
#include "oracle_common.h"

/* float atan2 in a FLOAT build (VelocityKernel.hpp:66-69 calls std::atan2 on
 * amrex::Real), double atan2 otherwise. */
static inline float orc_atan2_f32(float y, float x) { return atan2f(y, x); }
static inline double orc_atan2_f64(double y, double x) { return atan2(y, x); }

#define REAL double
#define FN(x) x##_f64
#include "oracle_fields.h"
#undef REAL
#undef FN

#define REAL float
#define FN(x) x##_f32
#include "oracle_fields.h"
#undef REAL
#undef FN

/* ---- exported scalar functions (ctypes) ---- */
int oracle_plaquette_winding(double t1, double t2, double t3, double t4)
{
    return orc_plaquette_winding(t1, t2, t3, t4);
}
double oracle_wrap_angle_diff(double d) { return orc_wrap_angle_diff(d); }

void oracle_plaquette_winding_batch(const double *th, int64_t n, int32_t *w)
{
    for (int64_t q = 0; q < n; ++q)
        w[q] = orc_plaquette_winding(th[4 * q], th[4 * q + 1], th[4 * q + 2], th[4 * q + 3]);
}

/* Background: out = {R, R', kappa, lambda, H, R2} at each tau. */
void oracle_background_eval(const orc_background *bg, const double *tau, int64_t n, double *out)
{
    for (int64_t q = 0; q < n; ++q) {
        double kap, lam, r2;
        orc_bg_rhs_coeffs(bg, tau[q], &kap, &lam, &r2);
        out[6 * q + 0] = orc_bg_R(bg, tau[q]);
        out[6 * q + 1] = orc_bg_R_prime(bg, tau[q]);
        out[6 * q + 2] = kap;
        out[6 * q + 3] = lam;
        out[6 * q + 4] = orc_bg_H(bg, tau[q]);
        out[6 * q + 5] = r2;
    }
}
double oracle_bg_H_over_mr_closed_form(const orc_background *bg, double tau)
{
    return orc_bg_H_over_mr_closed_form(bg, tau);
}
double oracle_bg_tau_from_log_mr_over_h(const orc_background *bg, double l)
{
    return orc_bg_tau_from_log_mr_over_h(bg, l);
}

double oracle_xi_from_comoving_length(double ell, double L, double a_inv, double tau)
{
    return orc_xi_from_comoving_length(ell, L, a_inv, tau);
}
double oracle_xi_from_plaquette_count(double N_p, double dx, double L, double a_inv, double tau)
{
    return orc_xi_from_plaquette_count(N_p, dx, L, a_inv, tau);
}
double oracle_plaquette_count_for_target_xi(double xi, int N, double L, double a_inv, double tau)
{
    return orc_plaquette_count_for_target_xi(xi, N, L, a_inv, tau);
}

double oracle_masking_weight(int scheme, double thr, double p1, double p2, double R)
{
    return orc_masking_weight(scheme, thr, p1, p2, R);
}
double oracle_masked_a_dot(int scheme, double thr, double p1, double p2, double q1, double q2,
                           double R)
{
    return orc_masked_a_dot(scheme, thr, p1, p2, q1, q2, R);
}

/* Energy pointwise functions: in = n x {psi1,psi2,Pi1,Pi2,g1sq,g2sq,gtsq,R,lambda,RpR},
 * out = n x {rho, a_kin(theta'), a_grad, r_kin, r_grad, r_mass}. */
void oracle_energy_pointwise(const double *in, int64_t n, double *out)
{
    for (int64_t q = 0; q < n; ++q) {
        const double *a = in + 10 * q;
        const double psi_sq = a[0] * a[0] + a[1] * a[1];
        const double thp = (psi_sq > 0.0) ? (a[0] * a[3] - a[2] * a[1]) / psi_sq : 0.0;
        out[6 * q + 0] = orc_rho_tot(a[0], a[1], a[2], a[3], a[4], a[5], a[7], a[8], a[9]);
        out[6 * q + 1] = orc_axion_kinetic(thp, a[7]);
        out[6 * q + 2] = orc_axion_gradient(a[6], a[7]);
        out[6 * q + 3] = orc_radial_kinetic(a[0], a[1], a[2], a[3], a[7], a[9]);
        out[6 * q + 4] = orc_radial_gradient(a[4], a[5], psi_sq, a[6], a[7]);
        out[6 * q + 5] = orc_radial_mass(a[0], a[1], a[7], a[8]);
    }
}

double oracle_gamma_sq_v_sq_from_phi(double a, double b, double c, double d, double m)
{
    return orc_gamma_sq_v_sq_from_phi(a, b, c, d, m);
}
double oracle_gamma_sq_v_sq_from_psi_literal(double a, double b, double c, double d, double R,
                                             double tau, double b_inv, double m)
{
    return orc_gamma_sq_v_sq_from_psi_literal(a, b, c, d, R, tau, b_inv, m);
}

/* FourierIC.hpp:82-116: fill the R2C half spectrum (nz, ny, nx/2+1) of one
 * component with hash-seeded Gaussian modes for 0 < k^2 <= k_max_cells^2
 * (integer mode indices, kx = i unwrapped, ky/kz wrapped), zero elsewhere.
 * spec is interleaved (re, im). The inverse FFT and the real-space rescale
 * (FourierIC.hpp:118-129) are done by the Python side of the oracle. */
void oracle_fourier_spectrum(double *spec, int nx, int ny, int nz, double k_max_cells,
                             uint64_t seed, int comp_seed_offset)
{
    const uint64_t full_seed = seed ^ ((uint64_t)comp_seed_offset << 32);
    const double kmax2 = k_max_cells * k_max_cells;
    const int nxh = nx / 2 + 1;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nxh; ++i) {
                const int kx = i, ky = orc_wrapped_freq(j, ny), kz = orc_wrapped_freq(k, nz);
                const double k2 = (double)(kx * kx + ky * ky + kz * kz);
                double re = 0.0, im = 0.0;
                if (!(k2 > kmax2 || k2 == 0.0)) orc_gaussian_mode(full_seed, 0, i, j, k, &re, &im);
                const int64_t o = 2 * (i + (int64_t)nxh * (j + (int64_t)ny * k));
                spec[o] = re;
                spec[o + 1] = im;
            }
}

uint64_t oracle_hash_u64(uint64_t x) { return orc_hash_u64(x); }

int oracle_sizeof_background(void) { return (int)sizeof(orc_background); }

/*
 * CPU oracle for the axion-string hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's per-level physics, used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker. It
 * is never linked into, or called by, the GPU library.
 *
 * Precision-independent pieces live here (plaquette winding, background
 * coefficient models, masking weight, energy/velocity pointwise formulas,
 * xi formula, Fourier-IC hash); the field loops are in oracle_fields.h, which
 * is instantiated once per precision by axs_oracle.c.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the reference project root).
 */
#ifndef AXS_ORACLE_COMMON_H
#define AXS_ORACLE_COMMON_H

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846

/* ---- plaquette winding: AxionStrings/PlaquetteWinding.hpp:24-51 ---- */
static inline double orc_wrap_angle_diff(double delta)
{
    const double pi = ORC_PI;
    const double two_pi = 2.0 * pi;
    delta = fmod(delta, two_pi);
    if (delta <= -pi)
        delta += two_pi;
    else if (delta > pi)
        delta -= two_pi;
    return delta;
}

static inline int orc_plaquette_winding(double t1, double t2, double t3, double t4)
{
    const double two_pi = 2.0 * ORC_PI;
    const double total = orc_wrap_angle_diff(t2 - t1) + orc_wrap_angle_diff(t3 - t2) +
                         orc_wrap_angle_diff(t4 - t3) + orc_wrap_angle_diff(t1 - t4);
    return (int)lround(total / two_pi);
}

/* ---- background coefficient models ----
 * Background.hpp:21-134 (power-law R(tau), c(tau) schedule, lambda re-anchored
 * at the switch), FlatBackground.hpp:26-44, PreEvolutionBackground.hpp:37-78,
 * and the optional post-handoff smoothstep blend of
 * AxionStringsLevel.cpp:893-906. `lambda_scale` multiplies lambda (the
 * reference hard-wires lambda0 = 1, Background.hpp:37; lambda is linear in
 * lambda0, so lambda_scale = lambda0 reproduces a general coupling). */
enum { ORC_BG_EXPANDING = 0, ORC_BG_FLAT = 1, ORC_BG_PRE = 2 };

typedef struct orc_background {
    int kind;            /* ORC_BG_* */
    double a_inv;        /* expanding: a ~ tau^(1/b_inv), b_inv = a_inv - 1 */
    double c0, c1, tau_switch;
    int has_switch;
    double lambda_scale; /* lambda0 multiplier (1 = reference convention) */
    double m_r;          /* flat background: lambda = m_r^2 */
    double gamma_pre;    /* pre-evolution: constant m_r/H */
    double blend_dtau;   /* > 0: post-handoff smoothstep blend active */
    double blend_tau_start, blend_lambda_start, blend_curv_start;
} orc_background;

static inline double orc_bg_b_inv(const orc_background *b) { return b->a_inv - 1.0; }
static inline double orc_bg_R0(const orc_background *b) { return 1.0 / (b->a_inv - 1.0); }

static inline double orc_bg_c(const orc_background *b, double tau)
{
    return (b->has_switch && tau >= b->tau_switch) ? b->c1 : b->c0; /* Background.hpp:28-31 */
}

static inline double orc_bg_R(const orc_background *b, double tau)
{
    if (b->kind == ORC_BG_FLAT) return 1.0;
    if (b->kind == ORC_BG_PRE) return exp(tau);
    return orc_bg_R0(b) * pow(tau / 1.0, 1.0 / orc_bg_b_inv(b)); /* Background.hpp:55-58 */
}

static inline double orc_bg_R_prime(const orc_background *b, double tau)
{
    if (b->kind == ORC_BG_FLAT) return 0.0;
    if (b->kind == ORC_BG_PRE) return exp(tau);
    const double b_inv = orc_bg_b_inv(b);
    return (orc_bg_R0(b) / (b_inv * 1.0)) * pow(tau / 1.0, 1.0 / b_inv - 1.0); /* :60-64 */
}

static inline double orc_bg_curvature(const orc_background *b, double tau)
{
    if (b->kind == ORC_BG_FLAT) return 0.0;
    if (b->kind == ORC_BG_PRE) return 1.0;
    const double b_inv = orc_bg_b_inv(b);
    return (1.0 - b_inv) / (b_inv * b_inv * tau * tau); /* Background.hpp:67-70 */
}

static inline double orc_bg_lambda_unit(const orc_background *b, double tau)
{
    if (b->kind == ORC_BG_FLAT) return b->m_r * b->m_r;
    if (b->kind == ORC_BG_PRE) {
        const double r = exp(tau);
        return b->gamma_pre * b->gamma_pre / (r * r); /* PreEvolutionBackground.hpp:62-66 */
    }
    /* Background.hpp:75-86 */
    const double lambda0 = 1.0;
    const double R0 = orc_bg_R0(b);
    const double c_now = orc_bg_c(b, tau);
    if (!b->has_switch || tau < b->tau_switch)
        return lambda0 * pow(orc_bg_R(b, tau) / R0, -2.0 * c_now);
    const double R_s = orc_bg_R(b, b->tau_switch);
    const double lambda_s = lambda0 * pow(R_s / R0, -2.0 * b->c0);
    return lambda_s * pow(orc_bg_R(b, tau) / R_s, -2.0 * c_now);
}

static inline double orc_bg_lambda(const orc_background *b, double tau)
{
    return b->lambda_scale * orc_bg_lambda_unit(b, tau);
}

static inline double orc_bg_H(const orc_background *b, double tau)
{
    const double R = orc_bg_R(b, tau);
    return orc_bg_R_prime(b, tau) / (R * R); /* Background.hpp:104-107 */
}

static inline double orc_bg_H_over_mr_closed_form(const orc_background *b, double tau)
{
    const double c_now = orc_bg_c(b, tau);
    return pow(tau / 1.0, (c_now - b->a_inv) / (b->a_inv - 1.0)); /* :92-96 */
}

static inline double orc_bg_tau_from_log_mr_over_h(const orc_background *b, double l)
{
    return 1.0 * exp(l * (b->a_inv - 1.0) / (b->a_inv - b->c0)); /* :129-133 */
}

/* RHS coefficients at conformal time tau (AxionStringsLevel.cpp:856-907). */
static inline void orc_bg_rhs_coeffs(const orc_background *b, double tau, double *kappa,
                                     double *lambda, double *R2)
{
    double k = orc_bg_curvature(b, tau);
    double l = orc_bg_lambda(b, tau);
    const double R = orc_bg_R(b, tau);
    if (b->kind == ORC_BG_EXPANDING && b->blend_dtau > 0.0) {
        const double t = (tau - b->blend_tau_start) / b->blend_dtau;
        if (t < 1.0) {
            const double tc = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
            const double s = tc * tc * (3.0 - 2.0 * tc);
            l = (1.0 - s) * b->blend_lambda_start + s * l;
            k = (1.0 - s) * b->blend_curv_start + s * k;
        }
    }
    *kappa = k;
    *lambda = l;
    *R2 = (b->kind == ORC_BG_FLAT) ? 1.0 : R * R;
}

/* ---- xi <-> plaquette count: AxionStrings/XiFormula.hpp:33-59 ---- */
static inline double orc_xi_from_comoving_length(double ell, double L, double a_inv, double tau)
{
    const double am1 = a_inv - 1.0;
    return ell / (L * L * L) * (am1 * am1 * am1 / (a_inv * a_inv)) * (tau * tau);
}

static inline double orc_xi_from_plaquette_count(double N_p, double dx, double L, double a_inv,
                                                 double tau)
{
    return orc_xi_from_comoving_length((2.0 / 3.0) * N_p * dx, L, a_inv, tau);
}

static inline double orc_plaquette_count_for_target_xi(double xi, int N, double L, double a_inv,
                                                       double tau)
{
    const double am1 = a_inv - 1.0;
    return 3.0 * N * xi * L * L * a_inv * a_inv / (2.0 * am1 * am1 * am1 * tau * tau);
}

/* ---- masking weight: AxionStrings/Masking.hpp:75-93 ---- */
enum { ORC_MASK_NONE = 0, ORC_MASK_A = 1, ORC_MASK_B = 2 };

static inline double orc_masking_weight(int scheme, double threshold, double psi1, double psi2,
                                        double R)
{
    if (scheme == ORC_MASK_NONE) return 1.0;
    const double mod = sqrt(psi1 * psi1 + psi2 * psi2) / R;
    if (scheme == ORC_MASK_B) return (mod >= threshold) ? 1.0 : 0.0;
    const double f_a = 1.4142135623730951;
    const double r = mod - 1.0;
    const double f = 1.0 + r / f_a;
    return f * f;
}

/* Masking.hpp:96-118 */
static inline double orc_masked_a_dot(int scheme, double threshold, double psi1, double psi2,
                                      double Pi1, double Pi2, double R)
{
    const double raw = psi1 * Pi2 - Pi1 * psi2;
    if (scheme == ORC_MASK_A) return raw;
    if (scheme == ORC_MASK_B && orc_masking_weight(scheme, threshold, psi1, psi2, R) == 0.0)
        return 0.0;
    const double psi_sq = psi1 * psi1 + psi2 * psi2;
    return raw / psi_sq;
}

/* ---- energy pointwise formulas: AxionStrings/Energy.hpp:64-190 ---- */
static inline double orc_rho_tot(double psi1, double psi2, double Pi1, double Pi2, double g1sq,
                                 double g2sq, double R, double lambda, double RpR)
{
    const double c1 = Pi1 - RpR * psi1;
    const double c2 = Pi2 - RpR * psi2;
    const double kinetic = c1 * c1 + c2 * c2;
    const double gradient = g1sq + g2sq;
    const double d = psi1 * psi1 + psi2 * psi2 - R * R;
    const double potential = 0.25 * lambda * d * d;
    const double R2 = R * R;
    return (kinetic + gradient + potential) / (R2 * R2);
}

static inline double orc_axion_kinetic(double theta_prime, double R)
{
    const double f_a = 1.4142135623730951;
    const double a_dot = f_a * theta_prime / R;
    return 0.5 * a_dot * a_dot;
}

static inline double orc_axion_gradient(double gtsq, double R)
{
    const double f_a = 1.4142135623730951;
    return 0.5 * f_a * f_a * gtsq / (R * R);
}

static inline double orc_radial_kinetic(double psi1, double psi2, double Pi1, double Pi2, double R,
                                        double RpR)
{
    const double c1 = Pi1 - RpR * psi1;
    const double c2 = Pi2 - RpR * psi2;
    const double psi_sq = psi1 * psi1 + psi2 * psi2;
    if (psi_sq <= 0.0) return 0.0;
    const double radial_dot = (psi1 * c1 + psi2 * c2) / sqrt(psi_sq);
    const double R2 = R * R;
    return (radial_dot * radial_dot) / (R2 * R2);
}

static inline double orc_radial_gradient(double g1sq, double g2sq, double psi_sq, double gtsq,
                                         double R)
{
    const double m = g1sq + g2sq - psi_sq * gtsq;
    const double R2 = R * R;
    return m / (R2 * R2);
}

static inline double orc_radial_mass(double psi1, double psi2, double R, double lambda)
{
    const double d = psi1 * psi1 + psi2 * psi2 - R * R;
    const double potential = 0.25 * lambda * d * d;
    const double R2 = R * R;
    return potential / (R2 * R2);
}

/* ---- string velocity: AxionStrings/Velocity.hpp:53-111 ---- */
static inline double orc_gamma_sq_v_sq_from_phi(double phi1, double phi2, double pd1, double pd2,
                                                double m_r)
{
    const double c1 = 0.41222, e1 = -0.025763;
    const double phi_sq = phi1 * phi1 + phi2 * phi2;
    const double pd_sq = pd1 * pd1 + pd2 * pd2;
    const double re = phi1 * pd1 + phi2 * pd2;
    const double m_r_sq = m_r * m_r;
    const double c1_sq = c1 * c1;
    const double term1 = (pd_sq / (2.0 * m_r_sq * c1_sq)) * (1.0 - e1 * phi_sq / (c1 * c1_sq));
    const double term2 = (e1 / (4.0 * m_r_sq * c1_sq * c1_sq * c1)) * re * re;
    return term1 - term2;
}

static inline double orc_gamma_sq_v_sq_from_psi_literal(double psi1, double psi2, double Pi1,
                                                        double Pi2, double R, double tau,
                                                        double b_inv, double m_r)
{
    const double c1 = 0.41222, e1 = -0.025763;
    const double bt = 1.0 / (b_inv * tau);
    const double d1 = Pi1 - bt * psi1, d2 = Pi2 - bt * psi2;
    const double diff_sq = d1 * d1 + d2 * d2;
    const double psi_sq = psi1 * psi1 + psi2 * psi2;
    const double re_term = (psi1 * Pi1 + psi2 * Pi2) - bt * psi_sq;
    const double R2 = R * R, R4 = R2 * R2, R6 = R4 * R2;
    const double m_r_sq = m_r * m_r, c1_sq = c1 * c1;
    const double term1 = (diff_sq / (2.0 * R4 * m_r_sq * c1_sq)) * (1.0 - e1 * psi_sq / (c1 * c1_sq * R2));
    const double term2 = (e1 / (4.0 * R6 * m_r_sq * c1_sq * c1_sq * c1)) * re_term * re_term;
    return term1 - term2;
}

/* ---- Fourier IC mode hash: AxionStrings/FourierIC.hpp:28-74 ---- */
static inline uint64_t orc_hash_u64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    x = x ^ (x >> 31);
    return x;
}

static inline double orc_uniform_from_hash(uint64_t h)
{
    return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

static inline void orc_gaussian_mode(uint64_t seed, int comp, int i, int j, int k, double *re,
                                     double *im)
{
    const uint64_t key = seed ^ ((uint64_t)comp << 60) ^ ((uint64_t)(uint32_t)i << 40) ^
                         ((uint64_t)(uint32_t)j << 20) ^ (uint64_t)(uint32_t)k;
    const uint64_t h1 = orc_hash_u64(key);
    const uint64_t h2 = orc_hash_u64(key ^ 0x1234567890ABCDEFULL);
    double u1 = orc_uniform_from_hash(h1);
    if (u1 < 1.0e-300) u1 = 1.0e-300;
    const double u2 = orc_uniform_from_hash(h2);
    const double r = sqrt(-2.0 * log(u1));
    const double theta = 2.0 * ORC_PI * u2;
    *re = r * cos(theta);
    *im = r * sin(theta);
}

static inline int orc_wrapped_freq(int idx, int n) { return (idx <= n / 2) ? idx : idx - n; }

/* ---- compensated (Neumaier) summation for the FP64 accumulations ---- */
typedef struct { double s, c; } orc_ksum;
static inline void orc_kadd(orc_ksum *a, double x)
{
    const double t = a->s + x;
    if (fabs(a->s) >= fabs(x))
        a->c += (a->s - t) + x;
    else
        a->c += (x - t) + a->s;
    a->s = t;
}
static inline double orc_kval(const orc_ksum *a) { return a->s + a->c; }

#endif

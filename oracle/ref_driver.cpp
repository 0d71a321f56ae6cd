// Driver that runs the reference's own hot-path headers on the host --
// TEST INFRASTRUCTURE ONLY (builds oracle/_ref/libaxs_ref_{f64,f32}.so).
//
// The headers are compiled unchanged from the reference tree (include path
// given by oracle/Makefile), against the project-written single-box AMReX
// shim in oracle/ref_shim/. This file only wires plain pointers into the
// reference's functions and exports them with C linkage; it restates no
// physics. The Makefile compiles it twice: amrex::Real = double and float.
#include "AxionStringsRHS.hpp"
#include "Background.hpp"
#include "Energy.hpp"
#include "EnergyKernel.hpp"
#include "FlatBackground.hpp"
#include "FourierIC.hpp"
#include "Masking.hpp"
#include "PlaquetteWinding.hpp"
#include "PreEvolutionBackground.hpp"
#include "StringFinder.hpp"
#include "StringTagger.hpp"
#include "MaskedFieldBuffer.hpp"
#include "SpectrumKernel.hpp"
#include "Velocity.hpp"
#include "VelocityKernel.hpp"
#include "XiFormula.hpp"

#include <cstdint>
#include <vector>

using amrex::Real;

namespace
{
amrex::MultiFab wrap_state(const Real *p, int nx, int ny, int nz, int ng)
{
    return amrex::MultiFab(const_cast<Real *>(p), nx, ny, nz, ng, 4);
}
MaskingParams masking(int scheme, double threshold)
{
    MaskingParams m{};
    m.scheme = scheme == 0 ? MaskingScheme::None : (scheme == 1 ? MaskingScheme::A : MaskingScheme::B);
    m.threshold = threshold;
    return m;
}
} // namespace

extern "C" {

int ref_real_size() { return int(sizeof(Real)); }

// AxionStringsRHS<FourthOrderDerivatives>::operator() over the valid cells,
// as AxionStringsLevel::specific_eval_rhs launches it (AxionStringsLevel.cpp:909-918).
void ref_rhs(const Real *soln, Real *rhs, int nx, int ny, int nz, int ng, double dx, double kappa,
             double lambda, double R2)
{
    auto s = wrap_state(soln, nx, ny, nz, ng);
    auto r = wrap_state(rhs, nx, ny, nz, ng);
    AxionStringsRHS<> op{static_cast<Real>(dx), static_cast<Real>(kappa), static_cast<Real>(lambda),
                        static_cast<Real>(R2)};
    const auto sa = s.const_arrays()[0];
    const auto ra = r.arrays()[0];
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) op(i, j, k, ra, sa);
}

// StringTagger::operator() (StringTagger.hpp:117-151) over the valid cells,
// as AxionStringsLevel::tag_cells launches it; tags[cell] = 1 where SET.
void ref_tag_cells(const Real *state, int nx, int ny, int nz, int ng, double dx, double gradient_threshold,
                   double radial_gradient_threshold, int8_t *tags)
{
    auto s = wrap_state(state, nx, ny, nz, ng);
    const auto a = s.const_arrays()[0];
    StringTaggerParams prm{};
    prm.gradient_threshold = gradient_threshold;
    prm.radial_gradient_threshold = radial_gradient_threshold;
    const StringTagger tagger(static_cast<Real>(dx), prm);
    std::vector<amrex::TagBox::TagType> t(size_t(nx) * ny * nz, amrex::TagBox::CLEAR);
    const amrex::Array4<amrex::TagBox::TagType> ta(t.data(), amrex::Dim3{0, 0, 0}, amrex::Dim3{nx, ny, nz}, 1);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) tagger(i, j, k, a, ta);
    for (size_t c = 0; c < t.size(); ++c) tags[c] = t[c] == amrex::TagBox::SET ? 1 : 0;
}

// fill_masked_a_dot_buffer (MaskedFieldBuffer.hpp) then compute_spectrum
// (SpectrumKernel.hpp:53-153) of the buffer, as specific_post_timestep
// does (AxionStringsLevel.cpp:1583-1640). shell_average/count are indexed by
// shell (0 where a shell is empty); out3 = {full_cube, inscribed_sphere,
// sum of buffer^2}; the buffer is written to `buf` (nx*ny*nz).
void ref_spectrum(const Real *state, int nx, int ny, int nz, int ng, int scheme, double threshold, double R,
                  double *shell_average, long *shell_count, double *out3, Real *buf)
{
    auto s = wrap_state(state, nx, ny, nz, ng);
    amrex::MultiFab b(amrex::BoxArray{amrex::Box{{nx, ny, nz}}}, amrex::DistributionMapping{}, 1, 0);
    fill_masked_a_dot_buffer(b, s, masking(scheme, threshold), static_cast<Real>(R));
    amrex::Geometry geom{amrex::Box{{nx, ny, nz}}};
    const Spectrum sp = compute_spectrum(b, geom);
    for (size_t q = 0; q < sp.p.size(); ++q) {
        const int shell = int(sp.p[q]);
        shell_average[shell] = sp.shell_average[q];
        shell_count[shell] = sp.shell_count[q];
    }
    out3[0] = sp.full_cube_energy;
    out3[1] = sp.inscribed_sphere_energy;
    out3[2] = double(amrex::MultiFab::Dot(b, 0, b, 0, 1, 0));
    const auto ba = b.array();
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) buf[i + size_t(nx) * (j + size_t(ny) * k)] = ba(i, j, k, 0);
}

void ref_windings(const Real *state, int nx, int ny, int nz, int ng, int8_t *w)
{
    auto s = wrap_state(state, nx, ny, nz, ng);
    const auto a = s.const_arrays()[0];
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const auto pw = plaquette_windings_at(a, i, j, k);
                const long cell = i + long(nx) * (j + long(ny) * k);
                w[3 * cell] = int8_t(pw.w_xy);
                w[3 * cell + 1] = int8_t(pw.w_yz);
                w[3 * cell + 2] = int8_t(pw.w_zx);
            }
}

void ref_count_plaquettes(const Real *state, int nx, int ny, int nz, int ng, const int *mask,
                          long *plain, long *weighted)
{
    auto s = wrap_state(state, nx, ny, nz, ng);
    amrex::iMultiFab m(const_cast<int *>(mask), nx, ny, nz, 0, 1);
    const auto c = count_plaquettes(s, mask ? &m : nullptr);
    *plain = c.n_p_plain;
    *weighted = c.n_p_weighted;
}

void ref_energy_sums(const Real *state, int nx, int ny, int nz, int ng, double dx, double R,
                     double lambda, double RpR, int scheme, double threshold, const int *mask,
                     double *out)
{
    auto s = wrap_state(state, nx, ny, nz, ng);
    amrex::iMultiFab m(const_cast<int *>(mask), nx, ny, nz, 0, 1);
    const auto e = compute_total_energy_sums(s, Real(dx), Real(R), Real(lambda), Real(RpR),
                                             masking(scheme, threshold), mask ? &m : nullptr);
    const double v[14] = {e.sum_rho,       e.sum_rho_w,      e.sum_rho_a_kin,  e.sum_rho_a_kin_w,
                          e.sum_rho_a_grad, e.sum_rho_a_grad_w, e.sum_rho_r_kin, e.sum_rho_r_kin_w,
                          e.sum_rho_r_grad, e.sum_rho_r_grad_w, e.sum_rho_r_mass, e.sum_rho_r_mass_w,
                          e.sum_w,         e.n_uncovered};
    for (int q = 0; q < 14; ++q) out[q] = v[q];
}

// compute_total_energy (EnergyKernel.hpp:239-268): out = {rho_u, rho_s, akin_u, akin_s,
// agrad_u, agrad_s, rkin_u, rkin_s, rgrad_u, rgrad_s, rmass_u, rmass_s, n_total, n_unmasked}.
void ref_total_energy(const Real *state, int nx, int ny, int nz, int ng, double dx, double R,
                      double lambda, double RpR, int scheme, double threshold, double *out)
{
    auto s = wrap_state(state, nx, ny, nz, ng);
    const auto e = compute_total_energy(s, Real(dx), Real(R), Real(lambda), Real(RpR),
                                        masking(scheme, threshold), long(nx) * ny * nz);
    const double v[14] = {e.rho_tot_unscreened,            e.rho_tot_screened,
                          e.rho_axion_kinetic_unscreened,  e.rho_axion_kinetic_screened,
                          e.rho_axion_gradient_unscreened, e.rho_axion_gradient_screened,
                          e.rho_radial_kinetic_unscreened, e.rho_radial_kinetic_screened,
                          e.rho_radial_gradient_unscreened, e.rho_radial_gradient_screened,
                          e.rho_radial_mass_unscreened,    e.rho_radial_mass_screened,
                          e.n_total,                       e.n_unmasked};
    for (int q = 0; q < 14; ++q) out[q] = v[q];
}

void ref_velocity(const Real *state, int nx, int ny, int nz, int ng, double R, double RpR,
                  double m_r, const int *mask, double *sum, long *count)
{
    auto s = wrap_state(state, nx, ny, nz, ng);
    amrex::iMultiFab m(const_cast<int *>(mask), nx, ny, nz, 0, 1);
    const auto v = compute_velocity_at_pierced_corners(s, Real(R), Real(RpR), Real(m_r), mask ? &m : nullptr);
    *sum = v.sum_gamma_sq_v_sq;
    *count = v.count;
}

// FourierIC::generate (FourierIC.hpp:82-130) into a ghost-free nx*ny*nz field.
void ref_fourier_ic(Real *field, int nx, int ny, int nz, double k_max_cells, double target_ms,
                    uint64_t seed, int comp_offset)
{
    amrex::MultiFab f(field, nx, ny, nz, 0, 1);
    amrex::Geometry geom{amrex::Box{{nx, ny, nz}}};
    FourierIC::generate(f, geom, k_max_cells, target_ms, seed, comp_offset);
}

uint64_t ref_hash_u64(uint64_t x) { return FourierIC::hash_u64(x); }

void ref_gaussian_mode(uint64_t seed, int comp, int i, int j, int k, double *re, double *im)
{
    FourierIC::gaussian_mode(seed, comp, i, j, k, *re, *im);
}

int ref_plaquette_winding(double a, double b, double c, double d) { return plaquette_winding(a, b, c, d); }
double ref_wrap_angle_diff(double d) { return wrap_angle_diff(d); }

// Background (Background.hpp:34-134): out = {R, R', curvature, lambda, H, H/m_r direct,
// H/m_r closed form} at tau.
void ref_background(double a_inv, double c0, double c1, double tau_switch, int has_switch,
                    double tau, double *out)
{
    CTauSchedule s{};
    s.c0 = c0;
    s.c1 = c1;
    s.tau_switch = tau_switch;
    s.has_switch = has_switch != 0;
    Background b(a_inv, s);
    out[0] = b.R(tau);
    out[1] = b.R_prime(tau);
    out[2] = b.curvature_term_coeff(tau);
    out[3] = b.lambda(tau);
    out[4] = b.H(tau);
    out[5] = b.H_over_mr_direct(tau);
    out[6] = b.H_over_mr_closed_form(tau);
}
double ref_tau_from_log_mr_over_h(double a_inv, double c0, double l)
{
    CTauSchedule s{};
    s.c0 = c0;
    return Background(a_inv, s).tau_from_log_mr_over_h(l);
}
void ref_flat_background(double m_r, double t, double *out)
{
    FlatBackground b(m_r);
    out[0] = b.R(t);
    out[1] = b.R_prime(t);
    out[2] = b.curvature_term_coeff(t);
    out[3] = b.lambda(t);
}
void ref_pre_background(double gamma_pre, double t, double *out)
{
    PreEvolutionBackground b(gamma_pre);
    out[0] = b.R(t);
    out[1] = b.R_prime(t);
    out[2] = b.curvature_term_coeff(t);
    out[3] = b.lambda(t);
    out[4] = b.m_r_over_H_direct(t);
}

double ref_xi_from_comoving_length(double ell, double L, double a_inv, double tau)
{
    return xi_from_comoving_length(ell, L, a_inv, tau);
}
double ref_xi_from_plaquette_count(double N_p, double dx, double L, double a_inv, double tau)
{
    return xi_from_plaquette_count(N_p, dx, L, a_inv, tau);
}
double ref_plaquette_count_for_target_xi(double xi, int N, double L, double a_inv, double tau)
{
    return plaquette_count_for_target_xi(xi, N, L, a_inv, tau);
}

double ref_masking_weight(int scheme, double thr, double p1, double p2, double R)
{
    return masking_weight(masking(scheme, thr), p1, p2, R);
}
double ref_masked_a_dot(int scheme, double thr, double p1, double p2, double q1, double q2, double R)
{
    return masked_a_dot(masking(scheme, thr), p1, p2, q1, q2, R);
}

// Energy.hpp pointwise: in = {psi1,psi2,Pi1,Pi2,g1sq,g2sq,gtsq,R,lambda,RpR},
// out = {rho, a_kin(theta'), a_grad, r_kin, r_grad, r_mass}.
void ref_energy_pointwise(const double *in, long n, double *out)
{
    for (long q = 0; q < n; ++q) {
        const double *a = in + 10 * q;
        const double psi_sq = a[0] * a[0] + a[1] * a[1];
        const double thp = (psi_sq > 0.0) ? (a[0] * a[3] - a[2] * a[1]) / psi_sq : 0.0;
        out[6 * q + 0] = rho_tot_pointwise(a[0], a[1], a[2], a[3], a[4], a[5], a[7], a[8], a[9]);
        out[6 * q + 1] = axion_kinetic_energy_pointwise(thp, a[7]);
        out[6 * q + 2] = axion_gradient_energy_pointwise(a[6], a[7]);
        out[6 * q + 3] = radial_kinetic_energy_pointwise(a[0], a[1], a[2], a[3], a[7], a[9]);
        out[6 * q + 4] = radial_gradient_energy_pointwise(a[4], a[5], psi_sq, a[6], a[7]);
        out[6 * q + 5] = radial_mass_energy_pointwise(a[0], a[1], a[7], a[8]);
    }
}

double ref_gamma_sq_v_sq_from_phi(double a, double b, double c, double d, double m)
{
    return gamma_sq_v_sq_from_phi(a, b, c, d, m);
}
double ref_gamma_sq_v_sq_from_psi_literal(double a, double b, double c, double d, double R,
                                          double tau, double b_inv, double m)
{
    return gamma_sq_v_sq_from_psi_literal(a, b, c, d, R, tau, b_inv, m);
}

} // extern "C"

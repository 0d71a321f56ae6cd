"""Background coefficient providers (host side), evaluated by the C library.

Mirrors the reference's analytic background classes:
``Background`` (AxionStrings/Background.hpp:21-134: R = R0 (tau/tau0)^(1/b_inv),
lambda = lambda0 (R/R0)^(-2c) with one re-anchored c-switch),
``FlatBackground`` (FlatBackground.hpp:26-44) and ``PreEvolutionBackground``
(PreEvolutionBackground.hpp:37-78), plus the post-handoff smoothstep blend of
AxionStringsLevel.cpp:893-906. ``lambda_scale`` multiplies lambda; the
reference fixes lambda0 = 1 (Background.hpp:37), which lambda_scale = 1 keeps.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import _lib as L


@dataclass(frozen=True)
class BackgroundValues:
    R: float
    R_prime: float
    kappa: float
    lambda_: float
    H: float
    R2: float
    m_r: float
    R_prime_over_R: float


@dataclass(frozen=True)
class Background:
    kind: int = L.BG_EXPANDING
    a_inv: float = 2.0
    c0: float = 0.0
    c1: float = 0.0
    tau_switch: float = 0.0
    has_switch: bool = False
    lambda_scale: float = 1.0
    m_r: float = 1.0
    gamma_pre: float = 1.0
    blend_dtau: float = 0.0
    blend_tau_start: float = 0.0
    blend_lambda_start: float = 0.0
    blend_curv_start: float = 0.0

    # -- constructors mirroring the reference classes --
    @classmethod
    def expanding(cls, a_inv: float = 2.0, c0: float = 0.0, *, c1: float = 0.0, tau_switch: float = 0.0,
                  has_switch: bool = False, lambda0: float = 1.0) -> "Background":
        return cls(L.BG_EXPANDING, a_inv, c0, c1, tau_switch, has_switch, lambda0)

    @classmethod
    def flat(cls, m_r: float = 1.0) -> "Background":
        return cls(kind=L.BG_FLAT, m_r=m_r)

    @classmethod
    def pre_evolution(cls, gamma_pre: float = 1.0) -> "Background":
        return cls(kind=L.BG_PRE_EVOLUTION, gamma_pre=gamma_pre)

    @property
    def b_inv(self) -> float:
        return self.a_inv - 1.0

    def to_c(self) -> L.BackgroundC:
        return L.BackgroundC(self.kind, int(self.has_switch), self.a_inv, self.c0, self.c1, self.tau_switch,
                             self.lambda_scale, self.m_r, self.gamma_pre, self.blend_dtau, self.blend_tau_start,
                             self.blend_lambda_start, self.blend_curv_start)

    def values(self, tau: float) -> BackgroundValues:
        v = L.BackgroundValues()
        L.call("axs_background_eval", C.byref(self.to_c()), float(tau), C.byref(v))
        return BackgroundValues(v.R, v.R_prime, v.kappa, v.lambda_, v.H, v.R2, v.m_r, v.R_prime_over_R)

    def rhs_coeffs(self, tau: float) -> L.RhsCoeffs:
        c = L.RhsCoeffs()
        L.call("axs_background_rhs_coeffs", C.byref(self.to_c()), float(tau), C.byref(c))
        return c

    # reference method names (Background.hpp)
    def R(self, tau: float) -> float:
        return self.values(tau).R

    def R_prime(self, tau: float) -> float:
        return self.values(tau).R_prime

    def curvature_term_coeff(self, tau: float) -> float:
        return self.values(tau).kappa

    def lambda_(self, tau: float) -> float:
        return self.values(tau).lambda_

    def H(self, tau: float) -> float:
        return self.values(tau).H

    def H_over_mr_direct(self, tau: float) -> float:
        v = self.values(tau)
        return v.H / v.m_r

    def tau_from_log_mr_over_h(self, log_mr_over_h: float) -> float:
        out = C.c_double()
        L.call("axs_background_tau_from_log_mr_over_h", C.byref(self.to_c()), float(log_mr_over_h), C.byref(out))
        return out.value


def xi_from_comoving_length(ell: float, L_tilde: float, a_inv: float, tau: float) -> float:
    """XiFormula.hpp:33-41."""
    return L.lib().axs_xi_from_comoving_length(ell, L_tilde, a_inv, tau)


def xi_from_plaquette_count(N_p: float, dx: float, L_tilde: float, a_inv: float, tau: float) -> float:
    """XiFormula.hpp:43-48."""
    return L.lib().axs_xi_from_plaquette_count(N_p, dx, L_tilde, a_inv, tau)


def plaquette_count_for_target_xi(xi: float, N: int, L_tilde: float, a_inv: float, tau: float) -> float:
    """XiFormula.hpp:52-58."""
    return L.lib().axs_plaquette_count_for_target_xi(xi, N, L_tilde, a_inv, tau)

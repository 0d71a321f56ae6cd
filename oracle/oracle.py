"""CPU oracle for the axion-string hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module. It loads

* ``oracle/_build/libaxs_oracle.so`` -- the plain-C restatement of the
  reference's per-level physics (axs_oracle.c), built by ``build()``;
* optionally ``oracle/_ref/libaxs_ref_{f64,f32}.so`` -- the reference's own
  hot-path headers compiled against a single-box AMReX shim, which exists only
  where the reference tree was available at build time. It pins the
  restatement.

Field arrays use the AMReX FArrayBox layout: shape ``(4, nz+2ng, ny+2ng,
nx+2ng)`` (component-major SoA, x fastest; AxionStringsRHS.impl.hpp:29-36).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libaxs_oracle.so")
REF_PATHS = {
    "f64": os.path.join(HERE, "_ref", "libaxs_ref_f64.so"),
    "f32": os.path.join(HERE, "_ref", "libaxs_ref_f32.so"),
}
# the reference project's root, where it exists (only the reference-built checker needs it)
REF_ROOT = os.environ.get("AXS_REFERENCE_DIR", "")
REF_SOURCE_DIR = os.path.join(REF_ROOT, "AxionStrings") if REF_ROOT else ""

_dbl = C.c_double
_i64 = C.c_int64
_ptr = C.c_void_p

BG_EXPANDING, BG_FLAT, BG_PRE = 0, 1, 2
MASK_NONE, MASK_A, MASK_B = 0, 1, 2


class OrcBackground(C.Structure):
    """Mirror of ``orc_background`` (oracle_common.h)."""

    _fields_ = [
        ("kind", C.c_int),
        ("a_inv", _dbl),
        ("c0", _dbl),
        ("c1", _dbl),
        ("tau_switch", _dbl),
        ("has_switch", C.c_int),
        ("lambda_scale", _dbl),
        ("m_r", _dbl),
        ("gamma_pre", _dbl),
        ("blend_dtau", _dbl),
        ("blend_tau_start", _dbl),
        ("blend_lambda_start", _dbl),
        ("blend_curv_start", _dbl),
    ]


def background(kind=BG_EXPANDING, a_inv=2.0, c0=0.0, c1=0.0, tau_switch=0.0, has_switch=False,
               lambda_scale=1.0, m_r=1.0, gamma_pre=1.0, blend_dtau=0.0, blend_tau_start=0.0,
               blend_lambda_start=0.0, blend_curv_start=0.0) -> OrcBackground:
    return OrcBackground(kind, a_inv, c0, c1, tau_switch, int(has_switch), lambda_scale, m_r,
                         gamma_pre, blend_dtau, blend_tau_start, blend_lambda_start,
                         blend_curv_start)


def build(force: bool = False) -> None:
    """Compile the C restatement (and, where AXS_REFERENCE_DIR names the
    reference tree, the reference-built checker) with oracle/Makefile."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    if REF_SOURCE_DIR and os.path.isdir(REF_SOURCE_DIR):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={REF_SOURCE_DIR}"], check=True)


_lib = None
_refs: dict = {}


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        for sfx in ("f64", "f32"):
            getattr(L, f"oracle_fill_periodic_{sfx}").argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
            getattr(L, f"oracle_rhs_{sfx}").argtypes = [_ptr, _ptr, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, _dbl, _dbl, _dbl]
            f = getattr(L, f"oracle_rk4_advance_{sfx}")
            f.argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, C.POINTER(OrcBackground), _dbl, _dbl, _dbl, C.c_int]
            f.restype = C.c_int
            getattr(L, f"oracle_count_plaquettes_{sfx}").argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, _ptr, C.POINTER(_i64), C.POINTER(_i64), _ptr]
            getattr(L, f"oracle_handoff_rescale_{sfx}").argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, _dbl, _dbl, _dbl]
            getattr(L, f"oracle_masked_a_dot_buffer_{sfx}").argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, _dbl, _ptr]
            getattr(L, f"oracle_tag_cells_{sfx}").argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, _dbl, _dbl, C.c_int, _ptr]
            getattr(L, f"oracle_energy_sums_{sfx}").argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, _dbl, _dbl, _dbl, C.c_int, _dbl, _ptr, _ptr]
            getattr(L, f"oracle_velocity_{sfx}").argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, _dbl, _dbl, _ptr, C.POINTER(_dbl), C.POINTER(_i64)]
        L.oracle_plaquette_winding.argtypes = [_dbl] * 4
        L.oracle_plaquette_winding.restype = C.c_int
        L.oracle_wrap_angle_diff.argtypes = [_dbl]
        L.oracle_wrap_angle_diff.restype = _dbl
        L.oracle_plaquette_winding_batch.argtypes = [_ptr, _i64, _ptr]
        L.oracle_background_eval.argtypes = [C.POINTER(OrcBackground), _ptr, _i64, _ptr]
        for name in ("oracle_bg_H_over_mr_closed_form", "oracle_bg_tau_from_log_mr_over_h"):
            getattr(L, name).argtypes = [C.POINTER(OrcBackground), _dbl]
            getattr(L, name).restype = _dbl
        for name, n in (("oracle_xi_from_comoving_length", 4), ("oracle_xi_from_plaquette_count", 5)):
            getattr(L, name).argtypes = [_dbl] * n
            getattr(L, name).restype = _dbl
        L.oracle_plaquette_count_for_target_xi.argtypes = [_dbl, C.c_int, _dbl, _dbl, _dbl]
        L.oracle_plaquette_count_for_target_xi.restype = _dbl
        L.oracle_masking_weight.argtypes = [C.c_int, _dbl, _dbl, _dbl, _dbl]
        L.oracle_masking_weight.restype = _dbl
        L.oracle_masked_a_dot.argtypes = [C.c_int] + [_dbl] * 6
        L.oracle_masked_a_dot.restype = _dbl
        L.oracle_energy_pointwise.argtypes = [_ptr, _i64, _ptr]
        L.oracle_gamma_sq_v_sq_from_phi.argtypes = [_dbl] * 5
        L.oracle_gamma_sq_v_sq_from_phi.restype = _dbl
        L.oracle_gamma_sq_v_sq_from_psi_literal.argtypes = [_dbl] * 8
        L.oracle_gamma_sq_v_sq_from_psi_literal.restype = _dbl
        L.oracle_fourier_spectrum.argtypes = [_ptr, C.c_int, C.c_int, C.c_int, _dbl, C.c_uint64, C.c_int]
        L.oracle_hash_u64.argtypes = [C.c_uint64]
        L.oracle_hash_u64.restype = C.c_uint64
        L.oracle_sizeof_background.restype = C.c_int
        assert L.oracle_sizeof_background() == C.sizeof(OrcBackground)
        _lib = L
    return _lib


def ref_available(prec: str = "f64") -> bool:
    return os.path.exists(REF_PATHS[prec])


def ref(prec: str = "f64"):
    """The reference's own headers compiled against the shim (None if absent)."""
    if prec in _refs:
        return _refs[prec]
    if not ref_available(prec):
        return None
    L = C.CDLL(REF_PATHS[prec])
    L.ref_real_size.restype = C.c_int
    L.ref_rhs.argtypes = [_ptr, _ptr, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, _dbl, _dbl, _dbl]
    L.ref_windings.argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, _ptr]
    L.ref_spectrum.argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, _dbl, _ptr, _ptr, _ptr, _ptr]
    L.ref_tag_cells.argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, _dbl, _dbl, _ptr]
    L.ref_count_plaquettes.argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, _ptr, C.POINTER(C.c_long), C.POINTER(C.c_long)]
    L.ref_energy_sums.argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, _dbl, _dbl, _dbl, C.c_int, _dbl, _ptr, _ptr]
    L.ref_total_energy.argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, _dbl, _dbl, _dbl, C.c_int, _dbl, _ptr]
    L.ref_velocity.argtypes = [_ptr, C.c_int, C.c_int, C.c_int, C.c_int, _dbl, _dbl, _dbl, _ptr, C.POINTER(_dbl), C.POINTER(C.c_long)]
    L.ref_fourier_ic.argtypes = [_ptr, C.c_int, C.c_int, C.c_int, _dbl, _dbl, C.c_uint64, C.c_int]
    L.ref_hash_u64.argtypes = [C.c_uint64]
    L.ref_hash_u64.restype = C.c_uint64
    L.ref_gaussian_mode.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(_dbl), C.POINTER(_dbl)]
    L.ref_plaquette_winding.argtypes = [_dbl] * 4
    L.ref_plaquette_winding.restype = C.c_int
    L.ref_wrap_angle_diff.argtypes = [_dbl]
    L.ref_wrap_angle_diff.restype = _dbl
    L.ref_background.argtypes = [_dbl, _dbl, _dbl, _dbl, C.c_int, _dbl, _ptr]
    L.ref_tau_from_log_mr_over_h.argtypes = [_dbl, _dbl, _dbl]
    L.ref_tau_from_log_mr_over_h.restype = _dbl
    L.ref_flat_background.argtypes = [_dbl, _dbl, _ptr]
    L.ref_pre_background.argtypes = [_dbl, _dbl, _ptr]
    for name, n in (("ref_xi_from_comoving_length", 4), ("ref_xi_from_plaquette_count", 5)):
        getattr(L, name).argtypes = [_dbl] * n
        getattr(L, name).restype = _dbl
    L.ref_plaquette_count_for_target_xi.argtypes = [_dbl, C.c_int, _dbl, _dbl, _dbl]
    L.ref_plaquette_count_for_target_xi.restype = _dbl
    L.ref_masking_weight.argtypes = [C.c_int, _dbl, _dbl, _dbl, _dbl]
    L.ref_masking_weight.restype = _dbl
    L.ref_masked_a_dot.argtypes = [C.c_int] + [_dbl] * 6
    L.ref_masked_a_dot.restype = _dbl
    L.ref_energy_pointwise.argtypes = [_ptr, C.c_long, _ptr]
    L.ref_gamma_sq_v_sq_from_phi.argtypes = [_dbl] * 5
    L.ref_gamma_sq_v_sq_from_phi.restype = _dbl
    L.ref_gamma_sq_v_sq_from_psi_literal.argtypes = [_dbl] * 8
    L.ref_gamma_sq_v_sq_from_psi_literal.restype = _dbl
    _refs[prec] = L
    return L


# ---------------------------------------------------------------- helpers
def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_ptr)


def _sfx(a: np.ndarray) -> str:
    if a.dtype == np.float64:
        return "f64"
    if a.dtype == np.float32:
        return "f32"
    raise TypeError(a.dtype)


def fab_shape(nx: int, ny: int, nz: int, ng: int, ncomp: int = 4):
    return (ncomp, nz + 2 * ng, ny + 2 * ng, nx + 2 * ng)


def to_fab(valid: np.ndarray, ng: int) -> np.ndarray:
    """(4, nz, ny, nx) -> FAB with ng periodic-filled ghosts."""
    c, nz, ny, nx = valid.shape
    f = np.zeros(fab_shape(nx, ny, nz, ng, c), dtype=valid.dtype)
    f[:, ng:ng + nz, ng:ng + ny, ng:ng + nx] = valid
    fill_periodic(f, ng)
    return f


def from_fab(f: np.ndarray, ng: int) -> np.ndarray:
    return np.ascontiguousarray(f[:, ng:f.shape[1] - ng, ng:f.shape[2] - ng, ng:f.shape[3] - ng])


def _dims(f: np.ndarray, ng: int):
    return f.shape[3] - 2 * ng, f.shape[2] - 2 * ng, f.shape[1] - 2 * ng


def fill_periodic(f: np.ndarray, ng: int) -> None:
    nx, ny, nz = _dims(f, ng)
    getattr(lib(), f"oracle_fill_periodic_{_sfx(f)}")(_p(f), nx, ny, nz, ng, f.shape[0])


# ------------------------------------------------------------ hot path
def rhs(soln: np.ndarray, ng: int, dx: float, kappa: float, lam: float, R2: float) -> np.ndarray:
    """AxionStringsRHS over the valid cells; ghosts of `soln` must be filled."""
    out = np.zeros_like(soln)
    nx, ny, nz = _dims(soln, ng)
    getattr(lib(), f"oracle_rhs_{_sfx(soln)}")(_p(soln), _p(out), nx, ny, nz, ng, dx, kappa, lam, R2)
    return out


def rk4_advance(state_fab: np.ndarray, ng: int, dx: float, bg: OrcBackground, tau_i: float,
                t0: float, dt: float, nsteps: int) -> None:
    """Classic RK4 (method of lines) in place on a FAB with ng >= 2."""
    nx, ny, nz = _dims(state_fab, ng)
    rc = getattr(lib(), f"oracle_rk4_advance_{_sfx(state_fab)}")(
        _p(state_fab), nx, ny, nz, ng, dx, C.byref(bg), tau_i, t0, dt, nsteps)
    if rc != 0:
        raise RuntimeError(f"oracle_rk4_advance failed ({rc})")


def count_plaquettes(state_fab: np.ndarray, ng: int, mask: np.ndarray | None = None,
                     want_windings: bool = False):
    nx, ny, nz = _dims(state_fab, ng)
    plain, weighted = _i64(0), _i64(0)
    w = np.zeros((nz, ny, nx, 3), dtype=np.int8) if want_windings else None
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
    getattr(lib(), f"oracle_count_plaquettes_{_sfx(state_fab)}")(
        _p(state_fab), nx, ny, nz, ng, None if m is None else _p(m), C.byref(plain),
        C.byref(weighted), None if w is None else _p(w))
    return (plain.value, weighted.value, w) if want_windings else (plain.value, weighted.value)


def handoff_rescale(state_fab: np.ndarray, ng: int, R_pre: float, R_pre_prime: float, R_main: float,
                    R_main_prime: float) -> None:
    """apply_pre_evolution_to_main_rescale on a FAB, in place (oracle_fields.h)."""
    nx, ny, nz = _dims(state_fab, ng)
    getattr(lib(), f"oracle_handoff_rescale_{_sfx(state_fab)}")(_p(state_fab), nx, ny, nz, ng, R_pre, R_pre_prime,
                                                                  R_main, R_main_prime)


def masked_a_dot_buffer(state_fab: np.ndarray, ng: int, scheme: int, threshold: float, R: float) -> np.ndarray:
    """fill_masked_a_dot_buffer (MaskedFieldBuffer.hpp:15-35): (nz, ny, nx) of the field precision."""
    nx, ny, nz = _dims(state_fab, ng)
    buf = np.zeros((nz, ny, nx), dtype=state_fab.dtype)
    getattr(lib(), f"oracle_masked_a_dot_buffer_{_sfx(state_fab)}")(
        _p(state_fab), nx, ny, nz, ng, scheme, threshold, R, _p(buf))
    return buf


def spectrum(buf: np.ndarray) -> dict:
    """compute_spectrum (SpectrumKernel.hpp:53-153) of a real (nz, ny, nx) field:
    unnormalised forward R2C (numpy's FFT in double; the reference's FFT runs in
    the field precision), then the reference's binning -- kx = 0 and kx = nx/2
    planes weight 1, others 2; shell = floor(|p| + 1/2) for |p| < n_max/2;
    shells accumulate w 4 pi |p|^2 |X|^2 and w. Returns per-shell sums
    (`shell_sum`, `shell_count`, index = shell) and the two totals."""
    nz, ny, nx = buf.shape
    X = np.fft.rfftn(buf.astype(np.float64), axes=(0, 1, 2))
    if buf.dtype == np.float32:
        X = X.astype(np.complex64).astype(np.complex128)
    n_max = max(nx, ny, nz)
    n_shells = n_max // 2 + 1
    kx = np.arange(nx // 2 + 1)
    ky = np.where(np.arange(ny) <= ny // 2, np.arange(ny), np.arange(ny) - ny)
    kz = np.where(np.arange(nz) <= nz // 2, np.arange(nz), np.arange(nz) - nz)
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    p_sq = (KX * KX + KY * KY + KZ * KZ).astype(np.float64)
    p = np.sqrt(p_sq)
    mag = X.real ** 2 + X.imag ** 2
    w = np.where((KX == 0) | (KX == nx // 2), 1.0, 2.0)
    full = float((w * mag).sum())
    ins = p < n_max / 2.0
    inscribed = float((w * mag)[ins].sum())
    shell = np.floor(p + 0.5).astype(np.int64)
    sel = ins & (shell < n_shells)
    shell_sum = np.bincount(shell[sel], weights=(w * 4.0 * np.pi * p_sq * mag)[sel], minlength=n_shells)
    shell_count = np.bincount(shell[sel], weights=w[sel], minlength=n_shells).astype(np.int64)
    return {"shell_sum": shell_sum, "shell_count": shell_count, "full_cube_energy": full,
            "inscribed_sphere_energy": inscribed}


def tag_cells(state_fab: np.ndarray, ng: int, dx: float, gradient_threshold: float = np.finfo(np.float64).max,
              radial_gradient_threshold: float = np.finfo(np.float64).max, n_error_buf: int = 0) -> np.ndarray:
    """StringTagger over the valid cells plus the periodic n_error_buf cube buffer:
    (nz, ny, nx) uint8 tags (oracle_fields.h: oracle_tag_cells)."""
    nx, ny, nz = _dims(state_fab, ng)
    tags = np.zeros((nz, ny, nx), dtype=np.uint8)
    getattr(lib(), f"oracle_tag_cells_{_sfx(state_fab)}")(
        _p(state_fab), nx, ny, nz, ng, dx, gradient_threshold, radial_gradient_threshold, n_error_buf, _p(tags))
    return tags


def energy_sums(state_fab: np.ndarray, ng: int, dx: float, R: float, lam: float, RpR: float,
                scheme: int = MASK_A, threshold: float = 0.8, mask=None) -> np.ndarray:
    nx, ny, nz = _dims(state_fab, ng)
    out = np.zeros(14)
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
    getattr(lib(), f"oracle_energy_sums_{_sfx(state_fab)}")(
        _p(state_fab), nx, ny, nz, ng, dx, R, lam, RpR, scheme, threshold,
        None if m is None else _p(m), _p(out))
    return out


def velocity(state_fab: np.ndarray, ng: int, R: float, RpR: float, m_r: float, mask=None):
    nx, ny, nz = _dims(state_fab, ng)
    s, c = _dbl(0), _i64(0)
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
    getattr(lib(), f"oracle_velocity_{_sfx(state_fab)}")(
        _p(state_fab), nx, ny, nz, ng, R, RpR, m_r, None if m is None else _p(m), C.byref(s),
        C.byref(c))
    return s.value, c.value


def normalise_energy(sums: np.ndarray, n_cells: float) -> np.ndarray:
    """compute_total_energy's single-level normalisation (EnergyKernel.hpp:239-268):
    {rho_u, rho_s, akin_u, akin_s, agrad_u, agrad_s, rkin_u, rkin_s, rgrad_u, rgrad_s,
     rmass_u, rmass_s, n_total, n_unmasked}."""
    out = np.zeros(14)
    sw = sums[12]
    for q in range(6):
        out[2 * q] = sums[2 * q] / n_cells
        out[2 * q + 1] = sums[2 * q + 1] / sw if sw > 0.0 else 0.0
    out[12] = n_cells
    out[13] = sw
    return out


def background_eval(bg: OrcBackground, taus) -> np.ndarray:
    t = np.ascontiguousarray(np.atleast_1d(taus), dtype=np.float64)
    out = np.zeros((t.size, 6))
    lib().oracle_background_eval(C.byref(bg), _p(t), t.size, _p(out))
    return out


def plaquette_winding_batch(theta: np.ndarray) -> np.ndarray:
    th = np.ascontiguousarray(theta, dtype=np.float64).reshape(-1, 4)
    w = np.zeros(th.shape[0], dtype=np.int32)
    lib().oracle_plaquette_winding_batch(_p(th), th.shape[0], _p(w))
    return w


# ------------------------------------------------------------ initial data
def fourier_spectrum(nx, ny, nz, k_max_cells, seed, comp_offset) -> np.ndarray:
    spec = np.zeros((nz, ny, nx // 2 + 1, 2))
    lib().oracle_fourier_spectrum(_p(spec), nx, ny, nz, k_max_cells, seed, comp_offset)
    return spec[..., 0] + 1j * spec[..., 1]


def fourier_ic_component(nx, ny, nz, k_max_cells, target_ms, seed, comp_offset) -> np.ndarray:
    """FourierIC::generate (FourierIC.hpp:82-130): seeded half spectrum, inverse
    real FFT with the FFTW c2r convention (numpy irfftn), real-space rescale to
    the target mean square. Returns a float64 (nz, ny, nx) field."""
    spec = fourier_spectrum(nx, ny, nz, k_max_cells, seed, comp_offset)
    field = np.fft.irfftn(spec, s=(nz, ny, nx), axes=(0, 1, 2))
    ms = float(np.dot(field.ravel(), field.ravel())) / field.size
    if ms > 0.0:
        field *= np.sqrt(target_ms / ms)
    return field


def fourier_ic_state(n: int, k_max_cells: float, seed: int, target_ms: float = 0.5,
                     dtype=np.float64) -> np.ndarray:
    """(4, n, n, n) state: psi1/psi2 from comp seeds 0/1 (AxionStringsLevel.cpp:810-815), Pi = 0."""
    s = np.zeros((4, n, n, n), dtype=dtype)
    s[0] = fourier_ic_component(n, n, n, k_max_cells, target_ms, seed, 0)
    s[1] = fourier_ic_component(n, n, n, k_max_cells, target_ms, seed, 1)
    return s


def strict_cutoff(n_max: float) -> float:
    """k_max_cells realising the strict |n| < n_max under the reference's
    inclusive rule k^2 <= k_max_cells^2 (integer k^2)."""
    return float(np.sqrt(n_max * n_max - 0.5))


@dataclass
class LevelDiagnostics:
    """Single-level subset of specific_post_timestep (AxionStringsLevel.cpp:1256-1362)."""
    n_p_plain: int
    n_p_weighted: int
    xi_plain: float
    xi_weighted: float
    energy: np.ndarray  # normalised, see normalise_energy
    energy_sums: np.ndarray
    vel_sum: float
    vel_count: int
    mean_gamma_sq_v_sq: float


def level_diagnostics(state_valid: np.ndarray, dx: float, bg: OrcBackground, tau: float,
                      scheme: int = MASK_A, threshold: float = 0.8) -> LevelDiagnostics:
    ng = 2
    fab = to_fab(np.ascontiguousarray(state_valid), ng)
    _, nz, ny, nx = state_valid.shape
    co = background_eval(bg, tau)[0]
    R, Rp, lam = co[0], co[1], co[3]
    RpR = Rp / R if bg.kind != BG_FLAT else 0.0
    m_r = float(np.sqrt(lam))
    plain, weighted = count_plaquettes(fab, ng)
    L = nx * dx
    a_inv = bg.a_inv
    xi_p = lib().oracle_xi_from_comoving_length((2.0 / 3.0) * plain * dx, L, a_inv, tau)
    xi_w = lib().oracle_xi_from_comoving_length((2.0 / 3.0) * weighted * dx, L, a_inv, tau)
    sums = energy_sums(fab, ng, dx, R, lam, RpR, scheme, threshold)
    vs, vc = velocity(fab, ng, R, RpR, m_r)
    mean = (vs * dx) / (vc * dx) if vc > 0 else 0.0
    return LevelDiagnostics(plain, weighted, xi_p, xi_w, normalise_energy(sums, float(nx * ny * nz)),
                            sums, vs, vc, mean)


def network_scalars_row(state_valid: np.ndarray, dx: float, bg: OrcBackground, tau: float,
                        scheme: int = MASK_A, threshold: float = 0.8) -> np.ndarray:
    """The 24 values of a network_scalars.dat row for one uncovered periodic
    level, restating specific_post_timestep's host algebra:

    * counts, comoving string lengths and the dx-weighted velocity sums of the
      composite gathering (AxionStringsLevel.cpp:1296-1340);
    * compute_composite_total_energy's volume-weighted normalisation
      (EnergyKernel.hpp:287-339) with a single level;
    * m_r/H from Background::H_over_mr_direct (AxionStringsLevel.cpp:1266-1269,
      Background.hpp:112-116);
    * <gamma^2 v^2>, <gamma>, the core energy, the axion tail and the two
      tensions (AxionStringsLevel.cpp:1358-1434);
    * the row order of AxionStringsLevel.cpp:1536-1579.
    """
    ng = 2
    fab = to_fab(np.ascontiguousarray(state_valid), ng)
    _, nz, ny, nx = state_valid.shape
    co = background_eval(bg, tau)[0]
    R, Rp, lam, H = co[0], co[1], co[3], co[4]
    RpR = Rp / R if bg.kind != BG_FLAT else 0.0
    m_r = float(np.sqrt(lam))
    m_r_over_h = 1.0 / (H / m_r)
    plain, weighted = count_plaquettes(fab, ng)
    L_tilde = nx * dx
    ell_p = (2.0 / 3.0) * float(plain) * dx
    ell_w = (2.0 / 3.0) * float(weighted) * dx
    xi_p = lib().oracle_xi_from_comoving_length(ell_p, L_tilde, bg.a_inv, tau)
    xi_w = lib().oracle_xi_from_comoving_length(ell_w, L_tilde, bg.a_inv, tau)
    vs, vc = velocity(fab, ng, R, RpR, m_r)
    v_sum, v_cnt = vs * dx, float(vc) * dx
    sums = energy_sums(fab, ng, dx, R, lam, RpR, scheme, threshold)
    vol = dx * dx * dx
    acc = [sums[q] * vol for q in range(12)]
    n_total = float(nx * ny * nz) * vol
    n_unmasked = sums[12] * vol
    e = [0.0] * 12
    for q in range(6):
        e[2 * q] = acc[2 * q] / n_total
        e[2 * q + 1] = acc[2 * q + 1] / n_unmasked if n_unmasked > 0.0 else 0.0
    mean_g2v2 = v_sum / v_cnt if v_cnt > 0.0 else 0.0
    mean_gamma = float(np.sqrt(1.0 + mean_g2v2))
    core = n_total * e[0] - n_unmasked * e[1]
    tail = n_unmasked * (e[5] - e[3])  # axion gradient minus axion kinetic, screened
    t_core = (R * R) * core / ell_p if ell_p > 0.0 else 0.0
    t_tail = (R * R) * (core + tail) / ell_p if ell_p > 0.0 else 0.0
    return np.array([plain, weighted, xi_p, xi_w, m_r_over_h] + e + [n_total, n_unmasked, mean_g2v2, mean_gamma,
                                                                     vc, t_core, t_tail], dtype=np.float64)

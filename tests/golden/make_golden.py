"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Runs the reference's unchanged hot-path headers (compiled by ``make -C oracle
ref`` into oracle/_ref/ against the single-box AMReX shim) on seeded inputs
and records inputs + outputs as compressed .npz files. Needs the reference
tree, so it only runs where that exists; the committed fixtures travel
instead.

    AXS_REFERENCE_DIR=<reference project root> python tests/golden/make_golden.py

Fixtures:
  kats.npz        known-answer vectors of the reference's own unit tests
                  (test_plaquette_winding.cpp, test_energy.cpp, test_velocity.cpp,
                  test_masking.cpp, test_background.cpp, test_xi_formula.cpp,
                  test_flat/pre_evolution_background.cpp) plus seeded random tuples
  fields_f64.npz  RHS, windings, plaquette counts (with/without coverage mask),
  fields_f32.npz  the 14 energy sums for schemes None/A/B, normalised energies,
                  velocity sum/count -- on a seeded random box and a seeded
                  Fourier-IC box, in the PRECISION=DOUBLE and =FLOAT builds
  fourier_ic.npz  FourierIC::generate outputs for two boxes / seeds
  spectrum.npz    fill_masked_a_dot_buffer + compute_spectrum shells and totals
  tagging.npz     StringTagger::operator() tags (plaquette, Laplacian and radial-
                  gradient criteria) on seeded boxes, both precision builds

    AXS_REFERENCE_DIR=<reference project root> python tests/golden/make_golden.py [fixture ...]   (default: all)
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def kats(R) -> dict:
    pi = np.pi
    out = {}
    # test_plaquette_winding.cpp:12-53 plus seeded random quadruples
    th = [
        (0.0, pi / 2, pi, 3 * pi / 2), (0.0, -pi / 2, -pi, -3 * pi / 2), (0.1, 0.2, 0.15, 0.05),
        (0.0, 0.0, 0.0, 0.0), (1.234, 1.234 + pi / 2, 1.234 + pi, 1.234 + 3 * pi / 2),
        (3.0, -3.0, 3.0, -3.0), (0.0, pi, 2 * pi, 3 * pi), (pi / 2, pi, 3 * pi / 2, 2 * pi),
    ]
    rng = np.random.default_rng(20261203)
    rand = rng.uniform(-pi, pi, size=(2000, 4))
    theta = np.concatenate([np.array(th), rand])
    out["winding_theta"] = theta
    out["winding_w"] = np.array([R.ref_plaquette_winding(*t) for t in theta], dtype=np.int32)
    d = np.concatenate([np.linspace(-7, 7, 57), [pi, -pi, 2 * pi, -2 * pi, 0.0]])
    out["wrap_in"] = d
    out["wrap_out"] = np.array([R.ref_wrap_angle_diff(x) for x in d])

    # Energy.hpp pointwise: test_energy.cpp tuples, vacuum points and random tuples
    rows = []
    for tau in (0.5, 1.0, 3.3, 10.0):  # vacuum psi = R, Pi = R' (a_inv = 2, c = 0)
        R_, Rp = tau, 1.0
        rows.append((R_, 0.0, Rp, 0.0, 0.0, 0.0, 0.0, R_, R_ ** 0, 1.0 / tau))
    for p in ((0.6, -0.3, 1.1, 0.4), (2.5, 1.8, -0.7, 2.2), (-1.2, 0.9, 0.05, -1.6)):
        rows.append((*p, 0.7, 1.3, 0.2, 1.9, 0.8, 1.0 / (1.7 * 2.3)))
    rows.append((0.0, 0.0, 1.0, -0.4, 0.7, 1.3, 0.0, 1.5, 0.8, 1.0 / (1.7 * 2.3)))
    rnd = rng.normal(size=(500, 10))
    rnd[:, 4:7] = np.abs(rnd[:, 4:7])
    rnd[:, 7] = np.abs(rnd[:, 7]) + 0.3
    rnd[:, 8] = np.abs(rnd[:, 8]) + 0.1
    e_in = np.ascontiguousarray(np.concatenate([np.array(rows), rnd]))
    e_out = np.zeros((e_in.shape[0], 6))
    R.ref_energy_pointwise(_p(e_in), e_in.shape[0], _p(e_out))
    out["energy_in"], out["energy_out"] = e_in, e_out

    # Masking.hpp (test_masking.cpp T2a points + random)
    m_in = []
    for scheme in (0, 1, 2):
        for p in ((0.2, 0.0, 0.3, -0.2), (1.5998, 0.0, 0.3, -0.2), (1.6, 0.0, 0.3, -0.2),
                  (1.6002, 0.0, 0.3, -0.2), (1.9, 0.4, -0.4, 0.5), (2.0, 0.0, 0.1, 0.1),
                  (0.075, 0.0, 0.2, -0.3)):
            m_in.append((scheme, 0.8, *p, 2.0))
        for r in rng.normal(size=(50, 4)):
            m_in.append((scheme, 0.8, *r, 1.3))
    m_in = np.array(m_in)
    out["mask_in"] = m_in
    out["mask_weight"] = np.array([R.ref_masking_weight(int(a[0]), *a[1:4], a[6]) for a in m_in])
    out["mask_adot"] = np.array([R.ref_masked_a_dot(int(a[0]), *a[1:]) for a in m_in])

    # Velocity.hpp (test_velocity.cpp points + random)
    pts = np.array([
        (0.3, -0.2, 0.05, 0.1, 1.0, 1.0, 1.0, 1.0), (0.3, -0.2, 0.05, 0.1, 2.0, 1.0, 1.0, 1.0),
        (0.3, -0.2, 0.05, 0.1, 2.0, 3.0, 1.0, 1.5), (-0.7, 0.4, -0.3, 0.2, 0.5, 2.0, 0.5, 0.8),
        (0.0, 0.9, 0.4, -0.1, 3.0, 4.0, 1.0, 1.0), (1.1, -1.1, 0.02, -0.02, 1.5, 0.7, 0.5, 2.0)])
    out["vel_psi_in"] = pts
    out["vel_psi_out"] = np.array([R.ref_gamma_sq_v_sq_from_psi_literal(*p) for p in pts])
    ph = rng.normal(size=(300, 5))
    ph[:, 4] = np.abs(ph[:, 4]) + 0.2
    out["vel_phi_in"] = ph
    out["vel_phi_out"] = np.array([R.ref_gamma_sq_v_sq_from_phi(*p) for p in ph])

    # Background.hpp: (a_inv, c0, c1, tau_switch, has_switch) x taus
    cfgs = np.array([(2.0, 0.0, 0, 0, 0), (2.0, 1.0, 0, 0, 0), (2.0, 2.0, 0, 0, 0),
                     (1.5, 0.0, 0, 0, 0), (3.0, 1.0, 0, 0, 0), (2.0, 1.0, 2.0, 5.0, 1),
                     (1.5, 1.0, 2.5, 2.0, 1)])
    taus = np.array([0.3, 0.5, 1.0, 2.7, 3.3, 4.999, 5.0, 5.001, 10.0, 12.3, 15.4])
    bg = np.zeros((len(cfgs), len(taus), 7))
    for a, c in enumerate(cfgs):
        for b, t in enumerate(taus):
            R.ref_background(c[0], c[1], c[2], c[3], int(c[4]), t, _p(bg[a, b]))
    out["bg_cfg"], out["bg_tau"], out["bg_out"] = cfgs, taus, bg
    logs = np.array([-2.0, -0.5, 0.0, 0.7, 3.1])
    out["bg_log_in"] = np.array([(a, c, l) for a in (1.5, 2.0, 3.0) for c in (0.0, 1.0) for l in logs])
    out["bg_log_tau"] = np.array([R.ref_tau_from_log_mr_over_h(*x) for x in out["bg_log_in"]])
    flat = np.zeros((3, 5, 4))
    pre = np.zeros((3, 5, 5))
    for a, m in enumerate((1.0, 2.3, 0.7)):
        for b, t in enumerate((0.0, 0.5, 1.0, 10.0, 100.0)):
            R.ref_flat_background(m, t, _p(flat[a, b]))
    for a, g in enumerate((0.5, 1.0, 3.0)):
        for b, t in enumerate((-2.0, -0.3, 0.0, 0.7, 4.0)):
            R.ref_pre_background(g, t, _p(pre[a, b]))
    out["flat_out"], out["pre_out"] = flat, pre

    # XiFormula.hpp
    xi_in = np.array([(12345.0, 0.05, 3.2, 2.0, 3.7), (987.0, 0.03, 4.2, 2.0, 5.5),
                      (2216.0, 0.5, 6.0, 2.0, 1.0), (100.0, 0.25, 8.0, 1.5, 2.0)])
    out["xi_in"] = xi_in
    out["xi_out"] = np.array([R.ref_xi_from_plaquette_count(*x) for x in xi_in])
    out["xi_len_out"] = np.array([R.ref_xi_from_comoving_length((2 / 3) * x[0] * x[1], *x[2:]) for x in xi_in])
    out["xi_inv_out"] = np.array([R.ref_plaquette_count_for_target_xi(0.7, 64, x[2], x[3], x[4]) for x in xi_in])
    return out


def fields(prec: str) -> dict:
    R = O.ref(prec)
    dt = np.float64 if prec == "f64" else np.float32
    out = {}
    rng = np.random.default_rng(77 if prec == "f64" else 78)
    ng = 2
    boxes = {
        # a rough random box (many pierced plaquettes) and a smooth Fourier-IC box
        "rand": (rng.standard_normal((4, 10, 11, 12)) * np.array([1, 1, 0.3, 0.3])[:, None, None, None]).astype(dt),
        "ic": np.concatenate([O.fourier_ic_state(16, 4.0, 4242)[:2],
                              0.2 * rng.standard_normal((2, 16, 16, 16))]).astype(dt),
    }
    params = dict(dx=0.5, kappa=-0.07, lam=1.3, R2=1.21, R=1.1, RpR=0.4, m_r=1.14)
    out["params"] = np.array([params[k] for k in ("dx", "kappa", "lam", "R2", "R", "RpR", "m_r")])
    for name, valid in boxes.items():
        _, nz, ny, nx = valid.shape
        fab = O.to_fab(np.ascontiguousarray(valid), ng)
        out[f"{name}_state"] = valid
        rhs = np.zeros_like(fab)
        R.ref_rhs(_p(fab), _p(rhs), nx, ny, nz, ng, params["dx"], params["kappa"], params["lam"], params["R2"])
        out[f"{name}_rhs"] = O.from_fab(rhs, ng)
        w = np.zeros((nz, ny, nx, 3), dtype=np.int8)
        R.ref_windings(_p(fab), nx, ny, nz, ng, _p(w))
        out[f"{name}_windings"] = w
        pl, wt = C.c_long(), C.c_long()
        R.ref_count_plaquettes(_p(fab), nx, ny, nz, ng, None, C.byref(pl), C.byref(wt))
        out[f"{name}_counts"] = np.array([pl.value, wt.value])
        mask = (rng.random((nz, ny, nx)) > 0.25).astype(np.int32)
        out[f"{name}_mask"] = mask.astype(np.uint8)
        R.ref_count_plaquettes(_p(fab), nx, ny, nz, ng, _p(mask), C.byref(pl), C.byref(wt))
        out[f"{name}_counts_masked"] = np.array([pl.value, wt.value])
        es = np.zeros((3, 14))
        et = np.zeros((3, 14))
        for scheme in (0, 1, 2):
            R.ref_energy_sums(_p(fab), nx, ny, nz, ng, params["dx"], params["R"], params["lam"],
                              params["RpR"], scheme, 0.8, None, _p(es[scheme]))
            R.ref_total_energy(_p(fab), nx, ny, nz, ng, params["dx"], params["R"], params["lam"],
                               params["RpR"], scheme, 0.8, _p(et[scheme]))
        em = np.zeros(14)
        R.ref_energy_sums(_p(fab), nx, ny, nz, ng, params["dx"], params["R"], params["lam"],
                          params["RpR"], 1, 0.8, _p(mask), _p(em))
        out[f"{name}_energy_sums"], out[f"{name}_energy_total"] = es, et
        out[f"{name}_energy_sums_masked"] = em
        s, c = C.c_double(), C.c_long()
        R.ref_velocity(_p(fab), nx, ny, nz, ng, params["R"], params["RpR"], params["m_r"], None,
                       C.byref(s), C.byref(c))
        out[f"{name}_velocity"] = np.array([s.value, float(c.value)])
    return out


def fourier() -> dict:
    R = O.ref("f64")
    out = {}
    for tag, (nx, ny, nz, kmax, seed, comp) in {"a": (16, 16, 16, 4.0, 4242, 0),
                                                 "b": (12, 10, 8, 3.2, 99, 1)}.items():
        f = np.zeros((nz, ny, nx))
        R.ref_fourier_ic(_p(f), nx, ny, nz, kmax, 0.5, seed, comp)
        out[f"{tag}_args"] = np.array([nx, ny, nz, kmax, seed, comp], dtype=np.float64)
        out[f"{tag}_field"] = f
    hin = np.array([0, 1, 2, 12345, 2 ** 63 + 7, 2 ** 64 - 1], dtype=np.uint64)
    out["hash_in"] = hin
    out["hash_out"] = np.array([R.ref_hash_u64(int(x)) for x in hin], dtype=np.uint64)
    return out


TAG_THRESHOLDS = [  # (gradient_threshold, radial_gradient_threshold); max = criterion off
    (np.finfo(np.float64).max, np.finfo(np.float64).max),
    (2.0, np.finfo(np.float64).max),
    (np.finfo(np.float64).max, 1.0),
    (4.0, 1.5),
]


def tagging() -> dict:
    """StringTagger::operator() (StringTagger.hpp:117-151) on the fields boxes
    of both precision builds, for the default (plaquette-only) criterion and
    with the Laplacian / radial-gradient criteria switched on."""
    out = {"thresholds": np.array(TAG_THRESHOLDS)}
    for prec in ("f64", "f32"):
        R = O.ref(prec)
        dt = np.float64 if prec == "f64" else np.float32
        rng = np.random.default_rng(91 if prec == "f64" else 92)
        boxes = {
            "rand": (rng.standard_normal((4, 10, 11, 12)) * np.array([1, 1, 0.3, 0.3])[:, None, None, None]).astype(dt),
            "ic": np.concatenate([O.fourier_ic_state(16, 4.0, 515)[:2],
                                  0.2 * rng.standard_normal((2, 16, 16, 16))]).astype(dt),
        }
        for name, valid in boxes.items():
            _, nz, ny, nx = valid.shape
            fab = O.to_fab(np.ascontiguousarray(valid), 2)
            out[f"{prec}_{name}_state"] = valid
            tags = np.zeros((len(TAG_THRESHOLDS), nz, ny, nx), dtype=np.int8)
            for t, (g, r) in enumerate(TAG_THRESHOLDS):
                R.ref_tag_cells(_p(fab), nx, ny, nz, 2, 0.5, g, r, _p(tags[t]))
            out[f"{prec}_{name}_tags"] = tags
    return out


def spectrum() -> dict:
    """fill_masked_a_dot_buffer + compute_spectrum (MaskedFieldBuffer.hpp,
    SpectrumKernel.hpp:53-153) on seeded boxes, schemes None and B, both
    precision builds (the shim's FFT is a direct DFT in double)."""
    out = {}
    for prec in ("f64", "f32"):
        R = O.ref(prec)
        dt = np.float64 if prec == "f64" else np.float32
        rng = np.random.default_rng(61 if prec == "f64" else 62)
        boxes = {"cube": (16, 16, 16), "odd": (12, 10, 8)}
        for name, (nx, ny, nz) in boxes.items():
            psi = [O.fourier_ic_component(nx, ny, nz, 3.0, 0.5, 808, c) for c in (0, 1)]
            v = np.concatenate([np.stack(psi), 0.3 * rng.standard_normal((2, nz, ny, nx))]).astype(dt)
            fab = O.to_fab(np.ascontiguousarray(v), 2)
            out[f"{prec}_{name}_state"] = v
            n_sh = max(nx, ny, nz) // 2 + 1
            for scheme in (0, 2):
                sa, sc, o3 = np.zeros(n_sh), np.zeros(n_sh, dtype=np.int64), np.zeros(3)
                buf = np.zeros((nz, ny, nx), dtype=dt)
                R.ref_spectrum(_p(fab), nx, ny, nz, 2, scheme, 0.8, 1.1, _p(sa), _p(sc), _p(o3), _p(buf))
                out[f"{prec}_{name}_s{scheme}_shell_average"] = sa
                out[f"{prec}_{name}_s{scheme}_shell_count"] = sc
                out[f"{prec}_{name}_s{scheme}_totals"] = o3
                out[f"{prec}_{name}_s{scheme}_buffer"] = buf
    return out


FIXTURES = {
    "kats": lambda: kats(O.ref("f64")),
    "fields_f64": lambda: fields("f64"),
    "fields_f32": lambda: fields("f32"),
    "fourier_ic": fourier,
    "tagging": tagging,
    "spectrum": spectrum,
}


def main(names=None) -> None:
    """Write the named fixtures (all by default)."""
    if not (O.ref_available("f64") and O.ref_available("f32")):
        O.build()
    if not (O.ref_available("f64") and O.ref_available("f32")):
        raise SystemExit("reference-built checker unavailable (set AXS_REFERENCE_DIR to the reference tree)")
    for name in names or FIXTURES:
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **FIXTURES[name]())
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1:])

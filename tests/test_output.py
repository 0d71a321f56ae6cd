"""Output tables and their restart semantics (no GPU): network_scalars.dat and
axion_spectrum.dat rows, the fresh-run move of an existing file, and the
restart trim of rows at or after the restart time (remove_duplicate_time_data);
the files load with the reference analysis loader's np.loadtxt layout."""
import os
import sys

import numpy as np
import pytest

from axion_strings_adaptive_gb300 import output as O
from axion_strings_adaptive_gb300.level import Diagnostics


def _diag(k):
    e = {f"{n}_{s}": 0.1 * k + i for i, n in enumerate(["rho_tot", "rho_axion_kinetic", "rho_axion_gradient",
                                                          "rho_radial_kinetic", "rho_radial_gradient",
                                                          "rho_radial_mass"]) for s in ("unscreened", "screened")}
    e.update(n_total=8.0, n_unmasked=7.5)
    return Diagnostics(n_p_plain=10 + k, n_p_weighted=11 + k, xi_plain=0.5, xi_weighted=0.6, energy=e,
                       energy_sums=[0.0] * 14, vel_sum=1.0, vel_count=4, mean_gamma_sq_v_sq=0.25, mean_gamma=1.1,
                       tension_core_only=3.0, tension_core_plus_tail=3.5, n_near_tie=0, n_listed=0)


def test_network_scalars_rows_and_restart(tmp_path):
    p = str(tmp_path / "network_scalars.dat")
    open(p, "w").write("stale\n")
    f = O.NetworkScalarsFile(p)
    assert any(n.startswith("network_scalars.dat.old.") for n in os.listdir(tmp_path))
    for k, tau in enumerate((1.0, 1.5, 2.0, 2.5)):
        f.write(tau, _diag(k), m_r_over_h=3.0 + k)
    data = np.loadtxt(p, comments="#")
    assert data.shape == (4, 1 + len(O.NETWORK_COLUMNS)) and len(O.NETWORK_COLUMNS) == 24
    assert data[2, 0] == 2.0 and data[2, 1] == 12 and data[2, 5] == 5.0
    # restart at tau = 2.0: rows from 2.0 on are redone
    f2 = O.NetworkScalarsFile(p, restart_tau=2.0)
    f2.write(2.0, _diag(9), m_r_over_h=1.0)
    data = np.loadtxt(p, comments="#")
    assert data[:, 0].tolist() == [1.0, 1.5, 2.0] and data[2, 1] == 19


def test_reference_loader_reads_our_tables(tmp_path):
    root = os.environ.get("AXS_REFERENCE_DIR", "")
    ref = os.path.join(root, "AxionStrings", "analysis")
    if not root or not os.path.isdir(ref):
        pytest.skip("AXS_REFERENCE_DIR does not name the reference tree (analysis scripts absent)")
    sys.path.insert(0, ref)
    try:
        import axion_analysis as A
    finally:
        sys.path.remove(ref)
    p = str(tmp_path / "network_scalars.dat")
    f = O.NetworkScalarsFile(p)
    f.write(1.25, _diag(0), 2.0)
    f.write(1.5, _diag(1), 2.5)  # (the loader needs two rows: np.loadtxt of one row is 1-D)
    cols = A.load_network_scalars(p)
    assert cols["tau"].tolist() == [1.25, 1.5] and cols["N_p"].tolist() == [10, 11]
    assert cols["m_r_over_H"].tolist() == [2.0, 2.5] and cols["tension_core_plus_tail"].tolist() == [3.5, 3.5]

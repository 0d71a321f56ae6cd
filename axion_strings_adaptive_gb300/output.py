"""Per-snapshot output files and checkpoints of the level path.

* ``network_scalars.dat`` (AxionStringsLevel.cpp:1541-1579): one row per
  snapshot, tau first, then the 24 columns of specific_post_timestep.
* ``axion_spectrum.dat`` (AxionStringsLevel.cpp:1692-1763): one row per shell
  per snapshot (tau, mode_index, k_over_H, then the screened / unscreened
  shell averages, totals and Parseval checks).

Both are whitespace-separated numeric tables with '#' header lines (the layout
the reference's analysis loader reads with ``np.loadtxt(comments="#")``). The
restart semantics are the reference's: a fresh run moves an existing file to
``<name>.old.<suffix>`` before writing its header; a restart at tau_r keeps the
file and first drops every row with tau >= tau_r (remove_duplicate_time_data),
so a redone segment does not duplicate rows.

Checkpoints (``save_checkpoint`` / ``load_checkpoint``) hold a level's valid
cells in its own precision plus the clock and background needed to resume.
"""
from __future__ import annotations

import dataclasses
import os
import secrets

import numpy as np
import torch

from .background import Background

NETWORK_COLUMNS = [
    "N_p", "N_p_weighted", "xi", "xi_weighted", "m_r_over_H",
    "rho_tot_unscreened", "rho_tot_screened",
    "rho_axion_kin_unscreened", "rho_axion_kin_screened",
    "rho_axion_grad_unscreened", "rho_axion_grad_screened",
    "rho_radial_kin_unscreened", "rho_radial_kin_screened",
    "rho_radial_grad_unscreened", "rho_radial_grad_screened",
    "rho_radial_mass_unscreened", "rho_radial_mass_screened",
    "n_total", "n_unmasked", "mean_gamma_sq_v_sq", "mean_gamma",
    "n_velocity_corners", "tension_core_only", "tension_core_plus_tail",
]

SPECTRUM_COLUMNS = [
    "shell_average_screened", "shell_average_unscreened",
    "full_cube_energy_screened", "full_cube_energy_unscreened",
    "inscribed_sphere_energy_screened", "inscribed_sphere_energy_unscreened",
    "real_space_mean_sq_screened", "real_space_mean_sq_unscreened",
    "parseval_full_screened", "parseval_full_unscreened",
    "parseval_inscribed_screened", "parseval_inscribed_unscreened",
]

_FMT = "%.10e"


class TableFile:
    """A time-keyed numeric table with '#' headers (first column: tau)."""

    def __init__(self, path: str, pre_columns: list, columns: list, restart_tau: float | None = None):
        self.path = path
        if restart_tau is None:
            if os.path.exists(path):
                os.replace(path, f"{path}.old.{secrets.token_hex(4)}")
            with open(path, "w") as f:
                f.write("# " + " ".join(pre_columns + columns) + "\n")
        else:
            self.remove_rows_from(restart_tau)

    def remove_rows_from(self, tau: float) -> None:
        """Drop every data row whose tau is >= `tau` (a restart redoes them)."""
        if not os.path.exists(self.path):
            return
        with open(self.path) as f:
            lines = f.readlines()
        keep = [ln for ln in lines if ln.startswith("#") or not ln.strip() or float(ln.split()[0]) < tau]
        with open(self.path, "w") as f:
            f.writelines(keep)

    def append(self, rows) -> None:
        with open(self.path, "a") as f:
            for r in rows:
                f.write(" ".join(_FMT % float(x) for x in r) + "\n")


def network_scalars_row(d, m_r_over_h: float) -> list:
    """The 24 values of one network_scalars.dat row from a Diagnostics."""
    e = d.energy
    return [d.n_p_plain, d.n_p_weighted, d.xi_plain, d.xi_weighted, m_r_over_h,
            e["rho_tot_unscreened"], e["rho_tot_screened"],
            e["rho_axion_kinetic_unscreened"], e["rho_axion_kinetic_screened"],
            e["rho_axion_gradient_unscreened"], e["rho_axion_gradient_screened"],
            e["rho_radial_kinetic_unscreened"], e["rho_radial_kinetic_screened"],
            e["rho_radial_gradient_unscreened"], e["rho_radial_gradient_screened"],
            e["rho_radial_mass_unscreened"], e["rho_radial_mass_screened"],
            e["n_total"], e["n_unmasked"], d.mean_gamma_sq_v_sq, d.mean_gamma,
            d.vel_count, d.tension_core_only, d.tension_core_plus_tail]


class NetworkScalarsFile(TableFile):
    def __init__(self, path: str, restart_tau: float | None = None):
        super().__init__(path, ["tau"], NETWORK_COLUMNS, restart_tau)

    def write(self, tau: float, d, m_r_over_h: float) -> None:
        self.append([[tau] + network_scalars_row(d, m_r_over_h)])


class AxionSpectrumFile(TableFile):
    def __init__(self, path: str, restart_tau: float | None = None):
        super().__init__(path, ["tau", "mode_index", "k_over_H"], SPECTRUM_COLUMNS, restart_tau)

    def write(self, tau: float, screened, unscreened) -> None:
        """One row per shell of two spectrum.Spectrum results (same binning)."""
        rows = []
        for q in range(len(screened.shell_average)):
            rows.append([tau, q, screened.k_over_H[q], screened.shell_average[q], unscreened.shell_average[q],
                         screened.full_cube_energy, unscreened.full_cube_energy,
                         screened.inscribed_sphere_energy, unscreened.inscribed_sphere_energy,
                         screened.real_space_mean_sq, unscreened.real_space_mean_sq,
                         screened.parseval_full, unscreened.parseval_full,
                         screened.parseval_inscribed, unscreened.parseval_inscribed])
        self.append(rows)


# ----------------------------------------------------------------------- checkpoints
def save_checkpoint(path: str, level, step: int = 0) -> None:
    """Valid cells of an AxionStringsLevel (its precision) plus its clock and background."""
    lv = level.level
    state = lv.get_state().cpu().numpy()
    bg = dataclasses.asdict(level.bg)
    np.savez(path, state=state, dx=lv.dx, tau_i=level.tau_i, time=level.time, step=step,
             background=np.array([bg[k] for k in sorted(bg)], dtype=np.float64),
             background_keys=np.array(sorted(bg)))


def load_checkpoint(path: str, level) -> int:
    """Restore a checkpoint into an AxionStringsLevel of the same shape; returns the step."""
    z = np.load(path)
    lv = level.level
    if tuple(z["state"].shape) != (4, lv.nz, lv.ny, lv.nx) or z["state"].dtype != np.dtype(
            torch.empty(0, dtype=lv.dtype).numpy().dtype):
        raise ValueError("checkpoint shape or precision does not match the level")
    lv.set_state(torch.from_numpy(z["state"]).to(lv.state.device))
    vals = dict(zip([str(k) for k in z["background_keys"]], z["background"].tolist()))
    for k in ("kind", "has_switch"):
        vals[k] = int(vals[k])
    vals["has_switch"] = bool(vals["has_switch"])
    level.bg = Background(**vals)
    level.tau_i = float(z["tau_i"])
    level.time = float(z["time"])
    return int(z["step"])

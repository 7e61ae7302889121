"""Pseudopotential containers (jrystal/pseudopotential/dataclass.py:23-200).

Unit conventions follow the reference: radial grids without r = 0, the
local potential and D matrices converted from Rydberg to Hartree (halved),
beta functions divided by r (UPF stores r beta(r)).  An element without
projectors gets one zero l = 0 beta and a zero 1 x 1 D matrix.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from .load import find_upf, parse_upf


@dataclass
class Pseudopotential:
  num_atom: int
  positions: np.ndarray
  charges: np.ndarray
  atomic_symbols: List[str]
  valence_charges: List[int]


@dataclass
class NormConservingPseudopotential(Pseudopotential):
  r_grid: List[np.ndarray]
  r_ab: List[np.ndarray]
  r_cutoff: List[Optional[float]]
  l_max: List[int]
  l_max_rho: List[Optional[int]]
  local_potential_grid: List[np.ndarray]
  local_potential_charge: List[int]
  num_beta: List[int]
  nonlocal_beta_grid: List[np.ndarray]
  nonlocal_beta_cutoff_radius: List
  nonlocal_d_matrix: List[np.ndarray]
  nonlocal_angular_momentum: List[np.ndarray]
  nonlocal_valence_configuration: List[List[dict]]

  @staticmethod
  def create(crystal, dir: Optional[str] = None) -> "NormConservingPseudopotential":
    """One entry per atom of ``crystal`` from the UPF files in ``dir``
    (dataclass.py:87-200)."""
    if dir is None:
      raise ValueError("a pseudopotential directory is required")
    fields = {k: [] for k in ("valence", "r", "rab", "rcut", "lmax", "lmax_rho", "vloc", "zloc",
                              "nbeta", "beta", "beta_rc", "dij", "angmom", "valconf")}
    for symbol in crystal.symbols:
      pp = parse_upf(find_upf(dir, symbol))
      hd = pp["PP_HEADER"]
      z = int(float(hd["z_valence"]))
      r_full = np.asarray(pp["PP_MESH"]["PP_R"], dtype=np.float64)
      keep = r_full > 0
      fields["valence"].append(z)
      fields["r"].append(r_full[keep])
      fields["rab"].append(np.asarray(pp["PP_MESH"]["PP_RAB"], dtype=np.float64)[keep])
      fields["rcut"].append(None)
      fields["lmax"].append(int(hd["l_max"]))
      fields["lmax_rho"].append(int(hd["l_max_rho"]) if "l_max_rho" in hd else None)
      fields["vloc"].append(np.asarray(pp["PP_LOCAL"], dtype=np.float64)[keep] / 2)
      fields["zloc"].append(z)
      betas = pp["PP_NONLOCAL"].get("PP_BETA")
      if betas:
        nb = len(betas)
        rb = np.stack([np.divide(np.asarray(b["values"], dtype=np.float64), r_full,
                                 out=np.zeros_like(r_full), where=keep) for b in betas])
        fields["nbeta"].append(nb)
        fields["beta"].append(rb[:, keep])
        fields["beta_rc"].append(betas[-1]["cutoff_radius"])
        d = np.asarray(pp["PP_NONLOCAL"]["PP_DIJ"], dtype=np.float64).reshape(nb, nb)
        fields["dij"].append(d / 2)
        fields["angmom"].append(np.array([int(b["angular_momentum"]) for b in betas]))
      else:
        fields["nbeta"].append(1)
        fields["beta"].append(np.zeros((1, int(keep.sum()))))
        fields["beta_rc"].append(0)
        fields["dij"].append(np.zeros((1, 1)))
        fields["angmom"].append(np.array([0]))
      fields["valconf"].append(pp["PP_INFO"]["Valence configuration"])
    f = fields
    return NormConservingPseudopotential(
      len(crystal.symbols), np.asarray(crystal.positions), np.asarray(crystal.charges),
      list(crystal.symbols), f["valence"], f["r"], f["rab"], f["rcut"], f["lmax"], f["lmax_rho"],
      f["vloc"], f["zloc"], f["nbeta"], f["beta"], f["beta_rc"], f["dij"], f["angmom"],
      f["valconf"])

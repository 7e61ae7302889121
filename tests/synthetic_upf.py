"""Analytic norm-conserving pseudopotentials written as UPF v2 files, for the
pseudopotential tests (test infrastructure; the values are model functions,
not fitted to any element):

  V_loc(r)  = -z erf(r / rc) / r                      (Hartree; file in Rydberg)
  beta_l(r) = r^l exp(-(r / w)^2)                     (file stores r beta(r))
  D         = diag(d)                                 (Hartree; file in Rydberg)

on the logarithmic mesh r_i = r0 exp(i dx) (plus r = 0 as the first point,
which the reader drops, as UPF meshes often start there).
"""
from __future__ import annotations

import os
from math import erf

import numpy as np


def write_upf(path, symbol, z_valence, betas=((0, 0.9), (1, 0.9)), dij=(0.8, 1.6), rc=0.8,
              r0=1e-3, dx=0.025, mesh=450, with_zero=True):
  r = r0 * np.exp(dx * np.arange(mesh))
  rab = r * dx
  if with_zero:
    r = np.concatenate([[0.0], r])
    rab = np.concatenate([[0.0], rab])
  safe = np.where(r > 0, r, 1.0)
  vloc_ha = np.where(r > 0, -z_valence * np.array([erf(x / rc) for x in r]) / safe,
                     -z_valence * 2 / (np.sqrt(np.pi) * rc))
  fmt = lambda a: "\n".join(" ".join(f"{v:.15e}" for v in a[i:i + 4]) for i in range(0, len(a), 4))
  nb = len(betas)
  lmax = max(l for l, _ in betas) if nb else -1
  info = "\n".join([
    "Generated by: synthetic_upf (analytic model)", "Author: tests", "Generation date: -",
    "Pseudopotential type: NC", f"Element: {symbol}", "Functional: SLA PZ",
    "Suggested minimum cutoff for wavefunctions: 10. Ry",
    "Suggested minimum cutoff for charge density: 40. Ry",
    "Scalar-relativistic calculation", "Local Potential: erf model",
    "Valence configuration:", "nl pn l occ Rcut Rcut US E pseu",
    f"3S 1 0 2.00 {rc:.3f} {rc:.3f} -0.5", "Generation configuration: none"])
  parts = [f'<UPF version="2.0.1">', f"<PP_INFO>\n{info}\n</PP_INFO>",
           f'<PP_HEADER element="{symbol}" pseudo_type="NC" relativistic="scalar" '
           f'is_ultrasoft="false" is_paw="false" core_correction="false" functional="SLA PZ" '
           f'z_valence="{float(z_valence):.12e}" l_max="{lmax}" mesh_size="{r.size}" '
           f'number_of_wfc="0" number_of_proj="{nb}"/>',
           f'<PP_MESH dx="{dx}" mesh="{r.size}" xmin="{np.log(r0):.6f}" rmax="{r[-1]:.6f}" zmesh="1.0">',
           f'<PP_R type="real" size="{r.size}" columns="4">\n{fmt(r)}\n</PP_R>',
           f'<PP_RAB type="real" size="{r.size}" columns="4">\n{fmt(rab)}\n</PP_RAB>', "</PP_MESH>",
           f'<PP_LOCAL type="real" size="{r.size}" columns="4">\n{fmt(2.0 * vloc_ha)}\n</PP_LOCAL>',
           "<PP_NONLOCAL>"]
  for i, (l, w) in enumerate(betas):
    rbeta = r * r ** l * np.exp(-(r / w) ** 2)
    parts.append(f'<PP_BETA.{i + 1} type="real" size="{r.size}" columns="4" index="{i + 1}" '
                 f'label="B{i + 1}" angular_momentum="{l}" cutoff_radius_index="{r.size}" '
                 f'cutoff_radius="{4 * w:.6f}" ultrasoft_cutoff_radius="0.0">\n{fmt(rbeta)}\n'
                 f"</PP_BETA.{i + 1}>")
  d = np.diag(np.asarray(dij, dtype=np.float64) * 2.0) if nb else np.zeros((1, 1))
  parts.append(f'<PP_DIJ type="real" size="{d.size}" columns="4">\n{fmt(d.reshape(-1))}\n</PP_DIJ>')
  parts += ["</PP_NONLOCAL>", "</UPF>"]
  with open(path, "w") as f:
    f.write("\n".join(parts) + "\n")
  return path


def write_set(directory, specs):
  """specs: {symbol: kwargs of write_upf}; returns the directory."""
  os.makedirs(directory, exist_ok=True)
  for sym, kw in specs.items():
    write_upf(os.path.join(directory, f"{sym}.synthetic.UPF"), sym, **kw)
  return directory

"""Crystal structure (jrystal/_src/crystal.py:34-189), atomic units inside."""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .const import ANGSTROM2BOHR, SYMBOL_TO_Z


@dataclass
class Crystal:
  """Charges, Cartesian positions (bohr), lattice vectors as rows (bohr)."""
  charges: np.ndarray
  positions: np.ndarray
  cell_vectors: np.ndarray
  spin: Optional[int] = None
  symbols: List[str] = field(default_factory=list)

  def __post_init__(self):
    self.charges = np.asarray(self.charges)
    self.positions = np.asarray(self.positions, dtype=np.float64).reshape(-1, 3)
    self.cell_vectors = np.asarray(self.cell_vectors, dtype=np.float64)
    if self.spin is None:
      self.spin = int(np.sum(self.charges)) % 2

  @property
  def scaled_positions(self):
    return self.positions @ np.linalg.inv(self.cell_vectors).T

  @property
  def vol(self):
    return float(abs(np.linalg.det(self.cell_vectors)))

  @property
  def num_atom(self):
    return self.positions.shape[0]

  @property
  def num_electron(self):
    return int(np.sum(self.charges))

  @property
  def A(self):
    return self.cell_vectors

  @property
  def reciprocal_vectors(self):
    return 2 * np.pi * np.linalg.inv(self.cell_vectors).T

  @property
  def B(self):
    return self.reciprocal_vectors

  @staticmethod
  def create_from_file(file_path: str, spin: Optional[int] = None) -> "Crystal":
    """Extended-xyz file (``Lattice="..."`` header, species and Cartesian Å)."""
    with open(file_path) as f:
      lines = f.read().splitlines()
    nat = int(lines[0].split()[0])
    header = lines[1]
    key = 'Lattice="'
    if key not in header:
      raise ValueError(f"{file_path}: no Lattice=\"...\" entry in the header line")
    i = header.index(key) + len(key)
    cell = np.array([float(v) for v in header[i:header.index('"', i)].split()]).reshape(3, 3)
    symbols, pos = [], []
    for ln in lines[2:2 + nat]:
      parts = ln.split()
      symbols.append(parts[0])
      pos.append([float(v) for v in parts[1:4]])
    charges = np.array([SYMBOL_TO_Z[s] for s in symbols])
    return Crystal(charges=charges, positions=np.array(pos) * ANGSTROM2BOHR,
                   cell_vectors=cell * ANGSTROM2BOHR, spin=spin, symbols=symbols)

  @staticmethod
  def create_from_symbols(symbols, positions, cell_vectors, spin: Optional[int] = None):
    """Symbols with Cartesian positions and cell in Å (as ase.Atoms takes them)."""
    if isinstance(symbols, str):
      import re
      symbols = [s for s, n in re.findall(r"([A-Z][a-z]?)(\d*)", symbols)
                 for _ in range(int(n) if n else 1)]
    charges = np.array([SYMBOL_TO_Z[s] for s in symbols])
    return Crystal(charges=charges, positions=np.asarray(positions) * ANGSTROM2BOHR,
                   cell_vectors=np.asarray(cell_vectors) * ANGSTROM2BOHR, spin=spin,
                   symbols=list(symbols))

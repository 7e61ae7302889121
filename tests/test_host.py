"""Host-side setup of the package (CPU): grids, masks, k-points, crystal
reader and the benchmark cells, checked against the oracle."""
import os

import numpy as np
import pytest

from oracle import restatement as R
from tests.systems import GOLDEN
from jrystal_gb300 import crystal, grid, workloads


def test_crystal_reader_matches_oracle():
  c = crystal.Crystal.create_from_file(os.path.join(GOLDEN, "diamond.xyz"))
  o = R.read_xyz(os.path.join(GOLDEN, "diamond.xyz"))
  np.testing.assert_array_equal(c.positions, o.positions)
  np.testing.assert_array_equal(c.cell_vectors, o.cell_vectors)
  assert c.spin == 0 and c.num_electron == 12
  np.testing.assert_allclose(c.reciprocal_vectors, o.reciprocal_vectors, rtol=1e-15)


@pytest.mark.parametrize("g", [(7, 8, 9), (16, 16, 16), (10, 12, 15)])
def test_grids_match_oracle(g):
  cell = R.read_xyz(os.path.join(GOLDEN, "diamond.xyz")).cell_vectors
  np.testing.assert_array_equal(grid.g_vectors(cell, g), R.g_vectors(cell, g))
  np.testing.assert_array_equal(grid.r_vectors(cell, g), R.r_vectors(cell, g))
  np.testing.assert_array_equal(grid.cubic_mask(g), R.cubic_mask(g))
  np.testing.assert_array_equal(grid.spherical_mask(cell, g, 20.0), R.spherical_mask(cell, g, 20.0))
  np.testing.assert_array_equal(grid.k_vectors(cell, (2, 3, 1)), R.k_vectors(cell, (2, 3, 1)))


def test_monkhorst_pack_convention():
  k = grid.monkhorst_pack((3, 3, 3))
  assert k.shape == (27, 3)
  assert np.any(np.all(k == 0, axis=1))            # odd grids contain Gamma
  np.testing.assert_allclose(grid.monkhorst_pack((2, 1, 1))[:, 0], [-0.25, 0.25])


def test_fft_sizes_and_proper_grid():
  assert grid.fft_factor(47) == 48 and grid.fft_factor(97) == 98
  assert list(grid.proper_grid_size(11)) == [12, 12, 12]
  with pytest.raises(ValueError):
    grid.fft_factor(4096)


def test_translation_vectors():
  cell = np.eye(3) * 10.0
  t = grid.translation_vectors(cell, 3000.0)
  n = int(np.ceil(3000.0 / np.linalg.norm(np.sum(cell, 0))**2))
  assert t.shape == (n**3, 3)
  np.testing.assert_array_equal(t, R.translation_vectors(cell, 3000.0))


@pytest.mark.parametrize("name,ng,nk", [("si2_fcc_48", 5029, 8), ("si8_cubic_64", 17071, 27),
                                         ("si64_supercell_96", 57747, 9)])
def test_benchmark_cells(name, ng, nk):
  wl = workloads.WORKLOADS[name]()
  assert int(wl.mask.sum()) == ng
  assert wl.kpts.shape == (nk, 3) and wl.num_kpt == nk
  occ = wl.occupation
  assert occ.shape == (1, nk, wl.num_band)
  assert abs(occ.sum() - 2 * wl.num_occ) < 1e-12
  wr, wi = wl.init_params()
  assert wr.shape == (1, nk, ng, wl.num_band)


def test_spin_channel_selection():
  """spin_restricted selects one or two channels; the polarised path is LDA
  only, so an unrestricted PBE run is refused before any device work."""
  from jrystal_gb300 import calc
  cfg = calc._merge({"xc": "lda_x+lda_c_vwn"})
  assert calc._num_spin(cfg) == 1
  cfg["spin_restricted"] = False
  assert calc._num_spin(cfg) == 2
  cfg["xc"] = "gga_x_pbe+gga_c_pbe"
  with pytest.raises(NotImplementedError):
    calc._num_spin(cfg)


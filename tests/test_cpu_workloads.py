"""Seeded synthetic workloads: subset-consistent, deterministic, and mapped as
stated (mol/L -> molecules/cm^3, H2O fixed). CPU only."""
import numpy as np

import simstack_gb300 as sg


def test_subset_consistency():
    """The first cells of a large batch are the same cells wherever they are generated."""
    a = sg.air_cells(4096, seed=1)
    b = sg.air_cells(96, seed=1)
    c = sg.air_cells(32, seed=1, first_cell=64)
    assert np.array_equal(a["y"][:, :96], b["y"][:, :96]) and np.array_equal(a["k"][:, :96], b["k"][:, :96])
    assert np.array_equal(a["y"][:, 64:96], c["y"][:, :32])


def test_distributions():
    z = sg.air_cells(8192, seed=3)
    y = z["y"][:, :8192] / sg.N_AVOGADRO_CM3
    assert np.all(y[16] == 55.5)                          # H2O
    lc = np.log10(y[:16])
    assert lc.min() >= -12.0 and lc.max() <= -2.0 and abs(lc.mean() + 7.0) < 0.05
    T = z.T[:8192]
    assert T.min() >= 288.0 and T.max() <= 303.0
    assert z.pH[:8192].min() >= 3.0 and z.pH[:8192].max() <= 7.0


def test_seed_changes_everything():
    assert not np.array_equal(sg.air_cells(64, seed=1)["y"], sg.air_cells(64, seed=2)["y"])


def test_padding_copies_cell_zero():
    z = sg.air_cells(13, seed=4)
    assert z.padded == 16 and np.array_equal(z["y"][:, 13], z["y"][:, 0])

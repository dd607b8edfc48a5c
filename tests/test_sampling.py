"""The frequency sampler without a GPU: the (bin, polarization) distribution the kernels draw
from their Walker alias tables equals the one Material::freqIndex's bisection draws from the
reference's own cumulative tables (psim/src/material.cpp:64-75), up to the tables' 21-bit
acceptance thresholds.

Reference distribution of a cumulative table cum[1000] with LA fractions la[1000]: the
bisection returns the first bin h >= 1 with u < cum[h] (bin 999 when there is none), so bin 1
takes cum[1], bin h in 2..998 takes cum[h] - cum[h-1] and bin 999 takes 1 - cum[998]; the bin is
LA with probability la[h] (TA when la[h] is NaN).  Kernel distribution of an alias table: a
32-bit word picks column c = word >> 21 (probability 1/2048) and keeps outcome c with
probability threshold / 2^21, else takes the alias outcome; outcome 2h is bin h LA, 2h + 1 bin
h TA, and outcomes beyond 1999 are clamped to 1999."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

COLS = 2048
ONE = float(1 << 21)


@pytest.fixture(scope="module")
def api(built):
    from psim_gb300 import api
    return api


def reference_distribution(table):
    cum, la = table[:, 0], table[:, 1]
    p = np.zeros(1000)
    p[1] = cum[1]
    p[2:999] = cum[2:999] - cum[1:998]
    p[999] = 1.0 - cum[998]
    p = np.maximum(p, 0.0)
    f = np.clip(np.nan_to_num(la, nan=0.0), 0.0, 1.0)
    out = np.zeros(2000)
    out[0::2] = p * f
    out[1::2] = p * (1.0 - f)
    return out / out.sum()


def kernel_distribution(words):
    thr = (words >> 11).astype(np.float64) / ONE
    alias = (words & 0x7FF).astype(np.int64)
    own = np.minimum(np.arange(COLS), 1999)
    out = np.zeros(2000)
    np.add.at(out, own, thr / COLS)
    np.add.at(out, np.minimum(alias, 1999), (1.0 - thr) / COLS)
    return out


def tables():
    for name in ("bar_ss", "bar_full", "kinked_small"):
        g = np.load(os.path.join(GOLDEN, f"tables_{name}.npz"))
        for kind in ("base", "emit", "scatter"):
            for i, t in enumerate(g["keep"]):
                yield f"{name}/{kind}/T={g['temps'][t]:.1f}", g[kind][i]


@pytest.mark.parametrize("label,table", list(tables()), ids=lambda v: v if isinstance(v, str) else "")
def test_alias_tables_sample_the_reference_distribution(api, label, table):
    words = api.alias_table(table)
    assert words.shape == (COLS,) and np.all((words & 0x7FF) < 2000)
    ref = reference_distribution(table)
    got = kernel_distribution(words)
    assert abs(got.sum() - 1.0) < 1e-12, label
    # each column's threshold is rounded to 2^-21, so an outcome is off by at most half a step
    # of 1/2048 for every column that can produce it
    bound = 0.5 / ONE / COLS * np.maximum(1, np.bincount(np.minimum((words & 0x7FF).astype(np.int64), 1999),
                                                           minlength=2000) + 1)
    assert np.all(np.abs(got - ref) <= bound + 1e-15), (label, np.max(np.abs(got - ref) / bound))
    # outcomes the reference never draws are never drawn
    assert np.all(got[ref == 0.0] == 0.0), label


def test_all_zero_table_draws_the_last_bin(api):
    """With every cumulative probability 0 the bisection never finds u < cum[h] and returns bin
    999; with an LA fraction of 0 it is TA.  The alias table draws that outcome only."""
    got = kernel_distribution(api.alias_table(np.zeros((1000, 2))))
    assert got[1999] == 1.0 and got[:1999].sum() == 0.0

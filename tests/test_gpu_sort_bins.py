"""The counting sort's large segments, in both forms.

The sort leaves every cell in ascending old index (the serial order of the reference's
counting sort, eng/particle_system.py:228-257).  Ordinary cells hold a few dozen particles;
a segment above 256 - here the out-of-grid bin after particles are moved far outside the
domain - takes the large-cell paths instead (a shared-memory sort up to 4,096 particles, a
scan over all particles above), which must give the same order, and the out-of-grid status
must still be raised.  Moved particles sit far to the left of the grid (x = -5 m), so their
flattened cell index is negative in either form's grid and they all land in the trailing
bin.
"""
import contextlib

import numpy as np
import pytest

from helpers import cfg_of, small_dambreak_2d

pytestmark = pytest.mark.gpu


def _expected_fp64(x, vs, grid, gnum, G):
    """Stable counting sort by flattened cell (truncating cast, x-major), out-of-grid
    particles in the trailing bin G, restated on the host."""
    t = (x - np.asarray(vs)[None, :]) / grid
    ok = np.all(np.abs(t) < 2147483647.0, axis=1)
    idx = np.where(ok[:, None], np.trunc(np.where(ok[:, None], t, 0.0)), 0).astype(np.int64)
    f = idx[:, 0] * gnum[1] * gnum[2] + idx[:, 1] * gnum[2] + idx[:, 2]
    f = np.where(ok & (f >= 0) & (f < G), f, G)
    return np.argsort(f, kind="stable")


@pytest.mark.parametrize("count", [1000, 6000])
def test_fp64_sort_out_of_grid_bin(native, count):
    from tisphi_gb300 import _native as nat
    from tisphi_gb300.simulation import Simulation

    sim = Simulation(cfg_of(small_dambreak_2d(spacing=0.005)), precision="fp64")
    ps = sim.ps
    cfg = ps._cfg
    fl = np.nonzero(ps.field("mat_type").cpu().numpy() == 1)[0]
    x = ps.field("x").cpu().numpy().astype(np.float64)
    rng = np.random.default_rng(count)
    moved = np.sort(rng.choice(fl, size=count, replace=False))
    x[moved, 0] = -5.0 - rng.random(count)
    id_before = ps.field("id0").cpu().numpy().copy()
    ps.write_field("x", np.ascontiguousarray(x))
    with contextlib.suppress(nat.NativeError):
        ps.initialize_particle_system()
    want = _expected_fp64(x, list(cfg.vdomain_start), float(cfg.grid_size), [int(v) for v in cfg.grid_num],
                          int(cfg.grid_num_total))
    np.testing.assert_array_equal(ps.field("id0").cpu().numpy(), id_before[want])
    # the moved particles end the order, in their previous order
    np.testing.assert_array_equal(ps.field("id0").cpu().numpy()[-count:], id_before[moved])
    with pytest.raises(nat.NativeError):
        ps.check_errors()


@pytest.mark.parametrize("count", [1000, 6000])
def test_fp32_sort_out_of_grid_bin(native, count):
    from tisphi_gb300 import _native as nat
    from tisphi_gb300.simulation import Simulation

    sim = Simulation(cfg_of(small_dambreak_2d(spacing=0.005)), precision="fp32_mixed")
    ps = sim.ps
    mt = ps.field("mat_type").cpu().numpy()
    nd = int(np.count_nonzero(mt == 1))  # the dynamic block: the fluid, stored first
    assert np.all(mt[:nd] == 1)
    x = ps.field("x").cpu().numpy().astype(np.float64)
    rng = np.random.default_rng(count)
    moved = np.sort(rng.choice(nd, size=count, replace=False))
    x[moved, 0] = -5.0 - rng.random(count)
    id_before = ps.field("id0").cpu().numpy().copy()
    ps.write_field("x", np.ascontiguousarray(x))
    with contextlib.suppress(nat.NativeError):
        ps.initialize_particle_system()
    ids = ps.field("id0").cpu().numpy()
    # the trailing bin closes the dynamic block: the moved particles in their previous order
    np.testing.assert_array_equal(ids[nd - count:nd], id_before[moved])
    # every other dynamic particle is still there, the static block untouched
    assert set(ids[:nd - count].tolist()) == set(np.delete(id_before[:nd], moved).tolist())
    np.testing.assert_array_equal(ids[nd:], id_before[nd:])
    with pytest.raises(nat.NativeError):
        ps.check_errors()

"""tsg_sort_noalloc: the cell-list sort for callers that cannot allocate device memory.

Callers whose device memory is planned up front (a fixed-budget pool, another framework's
allocator) or whose stepping loop must not risk the device-wide synchronisation of
cudaMalloc / cudaFree use this entry point; it keeps its scratch in fixed device arrays.
This file calls it through the C ABI twice in a row and checks both results against the
existing entry point, tsg_sort (particle order read back through id0, cell offsets
through tsg_grid).  Both outputs are integers, so they must match exactly, the bar every
sort test in this suite uses.  The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest


@pytest.mark.gpu
def test_noalloc_sort_matches_tsg_sort_on_two_calls(native):
    import torch

    from helpers import cfg_of, small_dambreak_2d
    from tisphi_gb300 import _native as nat
    from tisphi_gb300.simulation import Simulation

    lib = nat.load()
    sim = Simulation(cfg_of(small_dambreak_2d()))
    ps = sim.ps
    n = ps.particle_max_num
    G = ps.grid_num_total
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # caller-owned outputs
    cell_start = torch.empty(G + 2, dtype=torch.int32, device="cuda")
    perm = torch.empty(n, dtype=torch.int32, device="cuda")
    for call in range(2):
        x_before = ps.field("x").contiguous()  # (n, 3) row-major, current particle order
        id_before = ps.field("id0").cpu().numpy()
        rc = lib.tsg_sort_noalloc(ctypes.byref(ps._cfg), ctypes.c_void_p(x_before.data_ptr()), n,
                                  ctypes.c_void_p(cell_start.data_ptr()), ctypes.c_void_p(perm.data_ptr()), stream)
        assert rc == 0, f"call {call}: status {rc}"
        ps.initialize_particle_system()  # the existing entry point, tsg_sort
        torch.cuda.synchronize()
        id_after = ps.field("id0").cpu().numpy()
        p = perm.cpu().numpy()
        np.testing.assert_array_equal(id_before[p], id_after)
        cs = cell_start.cpu().numpy()
        np.testing.assert_array_equal(cs[1:G + 1], ps.grid_particle_num)
        assert cs[0] == 0 and cs[G + 1] == n
        sim.solver.step(5)  # move the particles so that the second call sorts a new input


def _expected_sort(x, vs, grid, gnum, G):
    """Stable counting sort by flattened cell (truncating cast, x-major), particles outside
    the grid or with non-finite positions in the trailing bin G: what the entry point must
    return, restated on the host."""
    with np.errstate(invalid="ignore"):
        t = (x - np.asarray(vs)[None, :]) / grid
    ok = np.all(np.abs(t) < 2147483647.0, axis=1)
    idx = np.where(ok[:, None], np.trunc(np.where(ok[:, None], t, 0.0)), 0).astype(np.int64)
    f = idx[:, 0] * gnum[1] * gnum[2] + idx[:, 1] * gnum[2] + idx[:, 2]
    f = np.where(ok & (f >= 0) & (f < G), f, G)
    perm = np.argsort(f, kind="stable").astype(np.int32)
    counts = np.bincount(f, minlength=G + 1)
    start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    return start, perm


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["3d", "outside_grid"])
def test_noalloc_sort_3d_grid_and_trailing_bin(native, case):
    """A 3D grid, and a 2D scene with particles moved outside the grid (one of them NaN):
    the trailing bin holds them in ascending index order, large enough to take both of the
    entry point's large-cell paths (a shared-memory sort, and a scan over all particles),
    on an explicit stream, twice in a row."""
    import torch

    from helpers import cfg_of, small_dambreak_2d, small_dambreak_3d
    from tisphi_gb300 import _native as nat
    from tisphi_gb300.simulation import Simulation

    lib = nat.load()
    d = small_dambreak_3d() if case == "3d" else small_dambreak_2d(spacing=0.005)
    ps = Simulation(cfg_of(d)).ps
    cfg = ps._cfg
    n = ps.particle_max_num
    G = int(cfg.grid_num_total)
    x = ps.field("x").cpu().numpy().astype(np.float64).copy()
    if case == "outside_grid":
        rng = np.random.default_rng(5)
        far = rng.choice(n, size=min(n - 100, 6000), replace=False)
        x[far, 0] = -5.0 - rng.random(far.size)  # left of the virtual domain
        x[far[:200], 1] = 1.0e3                   # far above it
        x[far[0], 2] = np.nan
    exp_start, exp_perm = _expected_sort(x, list(cfg.vdomain_start), float(cfg.grid_size),
                                         [int(v) for v in cfg.grid_num], G)
    if case == "outside_grid":
        assert exp_start[G + 1] - exp_start[G] > 4096  # the scan path; 200 took the other
    xd = torch.from_numpy(x).cuda().contiguous()
    side = torch.cuda.Stream()
    cell_start = torch.empty(G + 2, dtype=torch.int32, device="cuda")
    perm = torch.empty(n, dtype=torch.int32, device="cuda")
    with torch.cuda.stream(side):
        for call in range(2):
            perm.fill_(-1)
            rc = lib.tsg_sort_noalloc(ctypes.byref(cfg), ctypes.c_void_p(xd.data_ptr()), n,
                                      ctypes.c_void_p(cell_start.data_ptr()), ctypes.c_void_p(perm.data_ptr()),
                                      ctypes.c_void_p(side.cuda_stream))
            assert rc == 0, f"call {call}: status {rc}"
            side.synchronize()
            np.testing.assert_array_equal(cell_start.cpu().numpy(), exp_start)
            np.testing.assert_array_equal(perm.cpu().numpy(), exp_perm)


@pytest.mark.gpu
def test_noalloc_sort_rejects_sizes_beyond_its_scratch(native):
    import torch

    from helpers import cfg_of, small_dambreak_2d
    from tisphi_gb300 import _native as nat
    from tisphi_gb300.simulation import Simulation

    lib = nat.load()
    ps = Simulation(cfg_of(small_dambreak_2d())).ps
    x = ps.field("x").contiguous()
    out = torch.empty(8, dtype=torch.int32, device="cuda")
    too_many = 262144 + 1  # TSG_NOALLOC_MAX_PARTICLES + 1
    rc = lib.tsg_sort_noalloc(ctypes.byref(ps._cfg), ctypes.c_void_p(x.data_ptr()), too_many,
                              ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(out.data_ptr()), None)
    assert rc == -7  # TSG_E_CAPACITY, returned before any device work


def test_noalloc_sort_rejects_grid_beyond_its_scratch_without_gpu():
    """grid_num_total + 1 above TSG_NOALLOC_MAX_CELLS returns TSG_E_CAPACITY before any
    CUDA call, so this runs without a GPU (the pointers are never read)."""
    from tisphi_gb300 import _native as nat
    from tisphi_gb300 import build_native

    lib = ctypes.CDLL(build_native.build())
    cfg = nat.tsg_config()
    cfg.grid_size = 0.01
    cfg.grid_num[0], cfg.grid_num[1], cfg.grid_num[2] = 512, 512, 1
    cfg.grid_num_total = 512 * 512  # + 1 trailing bin = 262,145 > 262,144
    fake = ctypes.c_void_p(16)
    rc = lib.tsg_sort_noalloc(ctypes.byref(cfg), fake, ctypes.c_int64(1000), fake, fake, None)
    assert rc == -7  # TSG_E_CAPACITY
    cfg.grid_num[0] = 511  # within the limit: passes the size check, then needs a device
    assert lib.tsg_sort_noalloc(ctypes.byref(cfg), None, ctypes.c_int64(1000), fake, fake, None) == -1

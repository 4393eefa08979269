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

pytestmark = pytest.mark.gpu


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

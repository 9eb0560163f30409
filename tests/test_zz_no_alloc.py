"""bm_particle_contacts_static (scan workspace in a static device array) against
bm_particle_contacts on the same inputs, both called through the C-ABI.

The two entry points run the same kernels in the same order, so every output
of the pass (impulses, partner lists, bucket table, pair table, counters) must
be equal, bit for bit, on each of two calls in a row.  The static entry point must also leave the
solver's own scan partials untouched and allocate nothing (torch's allocator
and the device's free memory unchanged by a call).  The largest table has
2048 scan tiles, more than one chunk of the tile-sum scan.  This file is
collected last so it also runs after the other GPU tests have used the
library.
"""

import ctypes
from dataclasses import replace

import numpy as np
import pytest

from blademaster_gb300 import _native
from blademaster_gb300.solver import Config, Solver

pytestmark = pytest.mark.gpu

# Outputs whose layout is fixed by the inputs.  Slot positions inside the
# friction-history hash table and the order of particles inside one bucket
# depend on atomic arrival order, so those are compared as sets, and of the
# partner lists only the lanes in use (a list that overflowed its 64 lanes is
# marked -1 and its lanes are not read) are compared.
COMPARED = ("partner_count", "bucket_start", "particle_bucket", "particle_key", "pair_count", "flags")


def scene(cfg, seed):
    """Two solvers in one state: random sides of the cut, closing velocities, jittered positions."""
    solvers = [Solver(cfg), Solver(cfg)]
    rng = np.random.default_rng(seed)
    n = solvers[0].n
    x = solvers[0].reference + rng.normal(0.0, 0.1 * cfg.grid_spacing, (n, 3))
    v = rng.normal(0.0, 0.5, (n, 3))
    codes = rng.integers(0, 27, n).astype(np.int64)
    for s in solvers:
        s.x.assign(x)
        s.v.assign(v)
        s.codes.assign(codes)
        s.speed.fill_(1.0)
    return solvers


def partner_lists(solver):
    """The lanes in use of every partner list (zero elsewhere)."""
    partners = solver._t["partners"].cpu().numpy()
    count = solver._t["partner_count"].cpu().numpy()
    return np.where(np.arange(partners.shape[1])[None, :] < count[:, None], partners, 0)


def history_table(solver, table):
    """(keys, histories) of one friction-history table, sorted by key."""
    keys = solver._t["pair_keys"][table].cpu().numpy()
    history = solver._t["pair_history"][table].cpu().numpy()
    used = np.flatnonzero(keys >= 0)
    order = used[np.argsort(keys[used], kind="stable")]
    return keys[order], history[order]


def contacts(solver, entry, step):
    solver._flag("STEP", step)
    solver._flag("PAIR_DIRTY", 1)
    _native.check(getattr(solver._lib, entry)(solver._handle, solver._stream))


SENTINEL = -123457


@pytest.mark.parametrize("mode,spacing,tiles", [("list", 0.0075, 2), ("hash", 0.0075, 2), ("list", 0.0015, 256),
                                                ("hash", 0.0015, 256), ("list", 0.0008, 2048)])
def test_static_scratch_matches_particle_contacts_on_two_calls(mode, spacing, tiles):
    import torch

    cfg = replace(Config(), grid_spacing=spacing, pair_search=mode)
    existing, static = scene(cfg, seed=5)
    # 2048 tiles: more than one 1024-partial chunk per thread in the tile-sum scan
    assert static.buckets == 1024 * tiles
    # the solver's own scan partials (scratch words 64 .. 64 + tiles) must stay untouched
    own = static._t["scratch"][64 : 64 + tiles]
    own.fill_(SENTINEL)
    for step in range(2):
        contacts(existing, "bm_particle_contacts", step)
        existing.synchronize()
        static.synchronize()
        allocated, free = torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0]
        contacts(static, "bm_particle_contacts_static", step)
        static.synchronize()
        assert torch.cuda.memory_allocated() == allocated, f"call {step}"
        if step == 1:  # the first call may load the library's device code on this device
            assert torch.cuda.mem_get_info()[0] == free
        assert bool((own == SENTINEL).all()), f"call {step} wrote the solver's own scan partials"
        np.testing.assert_array_equal(static.impulses.numpy(), existing.impulses.numpy(), err_msg=f"call {step}")
        for name in COMPARED:
            np.testing.assert_array_equal(static._t[name].cpu().numpy(), existing._t[name].cpu().numpy(),
                                          err_msg=f"{name}, call {step}")
        np.testing.assert_array_equal(partner_lists(static), partner_lists(existing), err_msg=f"partners, call {step}")
        for table in range(2):
            a, b = (history_table(s, table) for s in (static, existing))
            np.testing.assert_array_equal(a[0], b[0], err_msg=f"pair keys {table}, call {step}")
            np.testing.assert_array_equal(a[1], b[1], err_msg=f"pair history {table}, call {step}")
    assert existing.pair_count[1].numpy()[0] > 0
    assert np.any(existing.impulses.numpy() != 0)


def test_static_scratch_rejects_a_table_beyond_its_size():
    solver = Solver(Config())
    lib = solver._lib
    params = solver._params
    too_big = _native.Params.from_buffer_copy(params)
    too_big.bucket_mask = 1024 * int(_native.header_constant("BM_STATIC_SCAN_PARTIALS")) * 2 - 1
    handle = ctypes.c_void_p()
    _native.check(lib.bm_solver_create(ctypes.byref(too_big), ctypes.byref(solver._buffers), ctypes.byref(handle)))
    try:
        rc = lib.bm_particle_contacts_static(handle, solver._stream)
        assert rc == 1 and b"more than 16,777,216 buckets" in lib.bm_last_error()
    finally:
        lib.bm_solver_destroy(handle)

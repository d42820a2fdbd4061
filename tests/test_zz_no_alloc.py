"""gbsph_sort_keys_noalloc -- the stable radix sort of the cell division run on
the library's fixed work area -- against the sort inside gbsph_divide (the
existing entry point): for the box keys of a divided case it must return the
same permutation and the same sorted keys, call after call, and it must refuse
sizes beyond its work area.  Integer work: the tolerance is exact equality.

The file is named to be collected last, and it also passes on its own.
"""
import ctypes as C
import tempfile

import numpy as np
import pytest

import goldens as G
from dualsphysics_gb300 import _lib
from dualsphysics_gb300 import casegen as cg
from dualsphysics_gb300.case import load_case
from dualsphysics_gb300.sph import GbSphSingle

pytestmark = pytest.mark.gpu


def _divided(cd):
    """The keys before sorting, the permutation and the sorted keys of the
    first divide (a full divide over [0, n)) of case `cd`."""
    s = GbSphSingle(0)
    s.setup(cd)
    n = len(cd.idp)
    perm = np.zeros(n, np.uint32)
    skeys = np.zeros(n, np.uint32)
    info = _lib.DivInfo()
    rc = _lib.lib().gbsph_get_divinfo(s.ctx, C.byref(info), None, 0, _lib.ptr(perm), _lib.ptr(skeys))
    assert rc == 0 and info.dividefull == 1 and info.np == n
    keys = np.empty(n, np.uint32)
    keys[perm] = skeys  # slot i of the sorted order holds the key of input index perm[i]
    return s, keys, perm, skeys


def _noalloc_sort(s, torch, keys, nbits):
    n = len(keys)
    d_keys = torch.from_numpy(keys.view(np.int32)).cuda()
    d_perm = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    d_sorted = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = _lib.lib().gbsph_sort_keys_noalloc(s.ctx, C.c_void_p(d_keys.data_ptr()), n, nbits,
                                            C.c_void_p(d_perm.data_ptr()), C.c_void_p(d_sorted.data_ptr()))
    assert rc == 0, _lib.lib().gbsph_last_error(s.ctx)
    s.sync()
    return d_perm.cpu().numpy().view(np.uint32)[:n], d_sorted.cpu().numpy().view(np.uint32)[:n]


def _c1():
    tmp = tempfile.mkdtemp(prefix="gbnoalloc_")
    spec = cg.spec_c1(name="DamC1")
    cg.write_case(cg.make_dam_break(spec), tmp)
    return load_case(tmp, "DamC1")


def test_noalloc_sort_equals_divide_sort_twice_in_a_row():
    torch = pytest.importorskip("torch")
    cases = [G.load_generated("mdbc_d04"), _c1(), G.load_generated("dbc_d04")]
    for cd in cases:
        s, keys, perm, skeys = _divided(cd)
        assert len(keys) <= _lib.SORT_NOALLOC_MAX_KEYS
        nbits = max(1, int(keys.max()).bit_length())
        for _ in range(2):  # two calls in a row on the same work area
            p, k = _noalloc_sort(s, torch, keys, nbits)
            np.testing.assert_array_equal(p, perm)
            np.testing.assert_array_equal(k, skeys)
        # a wider key width only adds passes over zero digits: same result
        p, k = _noalloc_sort(s, torch, keys, 32)
        np.testing.assert_array_equal(p, perm)
        s.close()


def test_noalloc_sort_refuses_what_it_cannot_do():
    torch = pytest.importorskip("torch")
    s, keys, _, _ = _divided(G.load_generated("dbc_d04"))
    d = torch.zeros(8, dtype=torch.int32, device="cuda")
    L = _lib.lib()
    ptr = C.c_void_p(d.data_ptr())
    rc = L.gbsph_sort_keys_noalloc(s.ctx, ptr, _lib.SORT_NOALLOC_MAX_KEYS + 1, 16, ptr, None)
    assert _lib.ERRORS[rc] == "GBSPH_ECAPACITY"
    assert b"exceed" in L.gbsph_last_error(s.ctx)
    assert _lib.ERRORS[L.gbsph_sort_keys_noalloc(s.ctx, ptr, 8, 0, ptr, None)] == "GBSPH_EINVAL"
    assert _lib.ERRORS[L.gbsph_sort_keys_noalloc(s.ctx, ptr, 8, 33, ptr, None)] == "GBSPH_EINVAL"
    assert _lib.ERRORS[L.gbsph_sort_keys_noalloc(s.ctx, ptr, 8, 16, None, None)] == "GBSPH_EINVAL"
    # a refused call leaves the context usable
    p, _ = _noalloc_sort(s, torch, np.array([3, 1, 2, 1], np.uint32), 2)
    np.testing.assert_array_equal(p, [1, 3, 2, 0])
    s.close()


def test_noalloc_sort_synthetic_sizes_and_no_device_allocation():
    """Against numpy's stable argsort at the edges of the work area: n = 0, 1,
    one 2048-key tile, and the maximum with many equal keys; after a warm-up
    call, further calls leave the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    s, _, _, _ = _divided(G.load_generated("dbc_d04"))
    rng = np.random.default_rng(7)
    _noalloc_sort(s, torch, np.array([5, 1], np.uint32), 3)      # warm-up (work area + kernels)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for n, nbits in ((0, 8), (1, 8), (2048, 13), (_lib.SORT_NOALLOC_MAX_KEYS, 10)):
        keys = rng.integers(0, 1 << nbits, size=n, dtype=np.uint64).astype(np.uint32)
        if n == _lib.SORT_NOALLOC_MAX_KEYS:
            keys = (keys % 97).astype(np.uint32)   # many ties
        d_keys = torch.from_numpy(keys.view(np.int32)).cuda() if n else torch.zeros(1, dtype=torch.int32,
                                                                                       device="cuda")
        d_perm = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
        d_sorted = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        for _ in range(2):
            rc = _lib.lib().gbsph_sort_keys_noalloc(s.ctx, C.c_void_p(d_keys.data_ptr()), n, nbits,
                                                    C.c_void_p(d_perm.data_ptr()), C.c_void_p(d_sorted.data_ptr()))
            assert rc == 0, _lib.lib().gbsph_last_error(s.ctx)
            s.sync()
            assert torch.cuda.mem_get_info()[0] == free_before      # the call allocated nothing
            if n:
                ref = np.argsort(keys, kind="stable").astype(np.uint32)
                np.testing.assert_array_equal(d_perm.cpu().numpy().view(np.uint32)[:n], ref)
                np.testing.assert_array_equal(d_sorted.cpu().numpy().view(np.uint32)[:n], keys[ref])
        del d_keys, d_perm, d_sorted
    assert free0 > 0
    s.close()

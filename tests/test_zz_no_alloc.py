"""bh_sort_keys_static: the sort entry point for callers that cannot allocate device memory.

Callers running inside a per-frame loop or a chain of stream callbacks cannot afford
cudaMalloc / cudaFree there (both synchronise the whole device), and embedders with a fixed
device-memory budget forbid allocations after start-up. This entry point sorts with scratch kept
in a fixed array of the library instead, for up to BH_SORT_STATIC_MAX_KEYS keys. The tests call
it through the C ABI, several times in a row on fresh keys (so every call starts from the
previous call's leftover scratch), and check its permutation exactly (integer output, so no
tolerance) against the oracle's stable sort and against the regular entry point
(bh_sort_bodies), across the sizes where the sort's code paths change: no key and one key
(copies only), a single partial tile, one key either side of a tile (4096 keys) and of the
regular path's rank-sort limit (16 384 keys), and the maximum. This file runs after every other
test, and it passes both on its own and after the rest of the suite.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 65536  # BH_SORT_STATIC_MAX_KEYS in include/bhgpu.h
SIZES = (0, 1, 2, 4095, 4097, 16384, 16385, 40001, MAX_KEYS)


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _static_sort(lib, torch, keys, vals, with_status=True):
    n = len(keys)
    kin = torch.from_numpy(keys.view(np.int64).copy()).cuda()
    vin = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    kout = torch.full_like(kin, -1)
    vout = torch.full_like(vin, -1)
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    ptr = (lambda t: t.data_ptr()) if n else (lambda t: None)
    rc = lib.bh_sort_keys_static(ptr(kin), ptr(vin), ptr(kout), ptr(vout), n, stream,
                                 status.data_ptr() if with_status else None)
    torch.cuda.synchronize()
    assert np.array_equal(kin.cpu().numpy().view(np.uint64), keys)  # inputs left unchanged
    st = int(status.item()) if with_status else 0
    return rc, kout.cpu().numpy().view(np.uint64), vout.cpu().numpy().view(np.uint32), st


def _morton_keys(sim, bh, seed, n):
    pm, v = bh.plummer(seed, n)
    sim.set_bodies(pm, v)
    _, size = sim.bounds()
    return sim.morton_keys(size)


def test_static_sort_matches_oracle_and_regular_sort(bh, orc):
    torch = _torch()
    lib = bh.load()
    with bh.Simulation(MAX_KEYS) as sim:
        for i, n in enumerate(SIZES):
            vals = np.arange(n, dtype=np.uint32)
            if n >= 2:
                keys = _morton_keys(sim, bh, 71 + i, n)
                perm = sim.sort_bodies()  # the regular entry point, on the same keys
            else:
                keys = (np.uint64(1) << np.uint64(63)) | np.arange(n, dtype=np.uint64)
                perm = None
            rc, ko, vo, status = _static_sort(lib, torch, keys, vals)
            assert rc == 0 and status == 0, (n, rc, status)
            ref = orc.sort_perm(keys)
            assert np.array_equal(vo, ref), n
            assert np.array_equal(ko, keys[ref]), n
            if perm is not None:
                assert np.array_equal(vo, perm), n


def test_static_sort_ties_and_no_status(bh, orc):
    """Many equal keys (stability decides the order), with caller values that are not indices,
    once with status_out and once without it."""
    torch = _torch()
    lib = bh.load()
    rng = np.random.default_rng(5)
    for n, with_status in ((MAX_KEYS, True), (30000, False), (4095, False)):
        keys = (np.uint64(1) << np.uint64(63)) | rng.integers(0, 300, n).astype(np.uint64) << np.uint64(40)
        vals = rng.permutation(n).astype(np.uint32)
        rc, ko, vo, status = _static_sort(lib, torch, keys, vals, with_status)
        assert rc == 0 and status == 0
        ref = orc.sort_perm(keys)
        assert np.array_equal(vo, vals[ref])
        assert np.array_equal(ko, keys[ref])


def test_static_sort_rejects_oversize(bh):
    lib = bh.load()
    assert lib.bh_sort_keys_static(None, None, None, None, MAX_KEYS + 1, None, None) == 1  # BH_ERR_INVALID_ARG

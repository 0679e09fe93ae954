"""bh_sort_keys_static: the sort entry point for callers that cannot allocate device memory.

Callers running inside a per-frame loop or a chain of stream callbacks cannot afford
cudaMalloc / cudaFree there (both synchronise the whole device), and embedders with a fixed
device-memory budget forbid allocations after start-up. This entry point sorts with scratch kept
in a fixed array of the library instead, for up to BH_SORT_STATIC_MAX_KEYS keys. The test calls
it through the C ABI twice in a row, each time on fresh keys, and checks that it reproduces the
permutation of the regular entry point (bh_sort_bodies) exactly (integer output, so no
tolerance). It lives in its own file so that it runs after every other test, and it passes both
on its own and after the rest of the suite.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 65536  # BH_SORT_STATIC_MAX_KEYS in include/bhgpu.h


def _static_sort(lib, torch, keys, vals):
    kin = torch.from_numpy(keys.view(np.int64).copy()).cuda()
    vin = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    kout = torch.empty_like(kin)
    vout = torch.empty_like(vin)
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.bh_sort_keys_static(kin.data_ptr(), vin.data_ptr(), kout.data_ptr(), vout.data_ptr(), len(keys),
                                 stream, status.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(kin.cpu().numpy().view(np.uint64), keys)  # inputs left unchanged
    return rc, kout.cpu().numpy().view(np.uint64), vout.cpu().numpy().view(np.uint32), int(status.item())


def test_static_sort_matches_regular_sort_twice(bh):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = bh.load()
    with bh.Simulation(MAX_KEYS) as sim:
        for seed, n in ((71, MAX_KEYS), (72, 40001)):
            pm, v = bh.plummer(seed, n)
            sim.set_bodies(pm, v)
            _, size = sim.bounds()
            keys = sim.morton_keys(size)
            perm = sim.sort_bodies()  # the regular entry point
            rc, ko, vo, status = _static_sort(lib, torch, keys, np.arange(n, dtype=np.uint32))
            assert rc == 0 and status == 0
            assert np.array_equal(vo, perm)
            assert np.array_equal(ko, keys[perm])


def test_static_sort_rejects_oversize(bh):
    lib = bh.load()
    assert lib.bh_sort_keys_static(None, None, None, None, MAX_KEYS + 1, None, None) == 1  # BH_ERR_INVALID_ARG

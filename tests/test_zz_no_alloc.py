"""The allocation-free diffusion entry point (ember_diffusion_integrate_noalloc).

It serves callers that must not allocate device memory while they step (an
application whose device memory belongs to another allocator, or code with a
footprint fixed at start-up): same results as ember_diffusion_integrate, with
the workspace in a fixed device array inside the library. Checked through the
C ABI against the allocating entry point, on two calls in a row (the array
keeps the previous call's contents), and for the size limit.

This file sorts last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from ember_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _case(seed, n_flames=4, n_vars=6):
    rng = np.random.default_rng(seed)
    grids, xs, Bs, Ds, Ss, Ys = [], [], [], [], [], []
    for f in range(n_flames):
        n = int(rng.integers(20, 300))
        dx = rng.uniform(1e-5, 1e-4) * np.exp(np.cumsum(rng.uniform(-0.3, 0.3, n - 1)))
        xs.append(np.concatenate([[0.0], dx]).cumsum())
        grids.append(L.DiffusionGrid(n, int(rng.integers(0, 5)), int(rng.choice([0, 1, 4])), int(rng.integers(0, 2))))
        Bs.append(np.exp(rng.uniform(-1, 1, n_vars * n)))
        Ds.append(np.exp(rng.uniform(np.log(1e-6), np.log(1e-3), n_vars * n)))
        Ss.append(rng.normal(scale=5.0, size=n_vars * n))
        Ys.append(np.cumsum(rng.normal(size=(n_vars, n)), axis=1).ravel())
    cat = np.concatenate
    return grids, n_vars, cat(xs), cat(Bs), cat(Ds), cat(Ss), cat(Ys)


def _run(torch, lib, fn_name, grids, n_vars, x, B, D, S, Y, t0, t1):
    dev = lambda a: torch.as_tensor(a, device="cuda")
    xd, Bd, Dd, Sd, Yd = dev(x), dev(B), dev(D), dev(S), dev(Y.copy())
    nsys = len(grids) * n_vars
    status = torch.full((nsys,), 99, dtype=torch.int32, device="cuda")
    garr = (L.DiffusionGrid * len(grids))(*grids)
    # the allocation-free entry point runs the serial algorithm; compare like with like
    opts = L.DiffusionOptions(t0, t1, 10.0, 2e-5, None, None, None, L.DIFFUSION_SERIAL)
    args = [len(grids), garr, n_vars, xd.data_ptr(), Bd.data_ptr(), Dd.data_ptr(), Sd.data_ptr(), Yd.data_ptr(),
            C.byref(opts), status.data_ptr()]
    if fn_name == "ember_diffusion_integrate":
        rc = lib.ember_diffusion_integrate(*args, L.MEM_DEVICE, None)
    else:
        rc = lib.ember_diffusion_integrate_noalloc(*args, None)
    torch.cuda.synchronize()
    assert rc == L.OK, L.last_error()
    return Yd.cpu().numpy(), status.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    lib = L.lib()
    assert lib.ember_device_count() >= 1
    for call, seed in enumerate((101, 202)):  # two calls in a row, different problems
        grids, n_vars, x, B, D, S, Y = _case(seed)
        ref, ref_status = _run(torch, lib, "ember_diffusion_integrate", grids, n_vars, x, B, D, S, Y, 0.0, 1e-5)
        out, status = _run(torch, lib, "ember_diffusion_integrate_noalloc", grids, n_vars, x, B, D, S, Y, 0.0, 1e-5)
        np.testing.assert_array_equal(status, ref_status)
        assert (status == 0).all()
        np.testing.assert_allclose(out, ref, rtol=1e-12, atol=0.0, err_msg=f"call {call + 1}")


def test_noalloc_call_leaves_device_memory_unchanged():
    # a warm call (the array's address already looked up, the kernels loaded)
    # changes neither the device's free memory nor torch's pools
    torch = pytest.importorskip("torch")
    lib = L.lib()
    grids, n_vars, x, B, D, S, Y = _case(303)
    dev = lambda a: torch.as_tensor(a, device="cuda")
    xd, Bd, Dd, Sd, Yd = dev(x), dev(B), dev(D), dev(S), dev(Y.copy())
    status = torch.zeros(len(grids) * n_vars, dtype=torch.int32, device="cuda")
    garr = (L.DiffusionGrid * len(grids))(*grids)
    opts = L.DiffusionOptions(0.0, 1e-5, 10.0, 2e-5, None, None, None, L.DIFFUSION_SERIAL)

    def call():
        rc = lib.ember_diffusion_integrate_noalloc(len(grids), garr, n_vars, xd.data_ptr(), Bd.data_ptr(),
                                                   Dd.data_ptr(), Sd.data_ptr(), Yd.data_ptr(), C.byref(opts),
                                                   status.data_ptr(), None)
        torch.cuda.synchronize()
        assert rc == L.OK, L.last_error()

    call()
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    call()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_reserved() == reserved0
    assert (status.cpu().numpy() == 0).all()


def test_noalloc_rejects_oversized_problem():
    lib = L.lib()
    n_vars = 8
    n = 70000  # 8 x 70000 = 560000 values > EMBER_NOALLOC_MAX_VALUES (524288)
    grids = (L.DiffusionGrid * 1)(L.DiffusionGrid(n, 0, 0, 0))
    opts = L.DiffusionOptions(0.0, 1e-5, 10.0, 2e-5, None, None, None, L.DIFFUSION_PARALLEL)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.ember_diffusion_integrate_noalloc(1, grids, n_vars, dummy, dummy, dummy, None, dummy, C.byref(opts),
                                               None, None)
    assert rc == L.EINVAL
    assert "exceed the maximum" in L.last_error()

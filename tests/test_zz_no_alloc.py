"""GPU test of gd_diag_static, the diagnostics entry point that allocates
no device memory, for callers that cannot call cudaMalloc (their device
memory belongs to another runtime's pool, or their budget is committed).

It must give the same answer as gd_diag, the context entry point that uses
allocated scratch, on the same fields, on two calls in a row (the second
call finds the shared scratch array holding the first call's contents).
Collected last so that a first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from gdpy import core, inputs

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_diag_static_matches_gd_diag_on_two_calls():
    torch = pytest.importorskip("torch")
    T, nlon, nlat, L = 42, 128, 64, 20
    ak, bk = inputs.hybrid_coords(L)
    g = core.Dycore(T, nlon, nlat, L, ak, bk, dt=1200.0)
    st = inputs.hs_rest_state(T, L, seed=5)
    g.set_state(st["vrt"], st["div"], st["tv"], st["lnps"])
    lib = core.load()
    dev = torch.device("cuda", 0)
    w = torch.from_numpy(g.grid_info()["gauwts"].copy()).to(dev)
    for step in range(2):
        g.advance(1)
        ref = g.diag()
        f = {k: torch.from_numpy(g.get_grid(k)).to(dev) for k in ("ug", "vg", "psg", "dlnpsdt")}
        out = torch.full((4,), -1.0, dtype=torch.float64, device=dev)
        s = torch.cuda.current_stream()
        rc = lib.gd_diag_static(_ptr(f["ug"]), _ptr(f["vg"]), L, _ptr(f["psg"]), _ptr(f["dlnpsdt"]), _ptr(w),
                                nlat, nlon, _ptr(out), ctypes.c_void_p(s.cuda_stream))
        assert rc == core.GD_OK
        torch.cuda.synchronize()
        o = out.cpu().numpy()
        want = np.array([ref["spdmax"], ref["psmin"], ref["psmax"], ref["pstend"]])
        np.testing.assert_allclose(o, want, rtol=1e-12, atol=0)
        assert want[0] > 0 and want[3] > 0


def test_diag_static_rejects_oversized_and_null_arguments():
    lib = core.load()
    p = ctypes.c_void_p(8)  # never dereferenced: the size check comes first
    assert lib.gd_diag_static(p, p, 4, p, p, p, 4097, 16, p, None) == core.GD_ERR_ARG
    assert lib.gd_diag_static(None, p, 4, p, p, p, 64, 16, p, None) == core.GD_ERR_ARG

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


_RESET_SCRIPT = r"""
import ctypes, sys
import numpy as np
from gdpy import core
lib = core.load()
rt = ctypes.CDLL("libcudart.so.13")
vp = ctypes.c_void_p
rt.cudaMalloc.argtypes = [ctypes.POINTER(vp), ctypes.c_size_t]
rt.cudaMemcpy.argtypes = [vp, vp, ctypes.c_size_t, ctypes.c_int]
rt.cudaFree.argtypes = [vp]
H2D, D2H = 1, 2
nlev, nlat, nlon = 3, 32, 64
rng = np.random.default_rng(7)
host = dict(ug=rng.standard_normal((nlev, nlat, nlon)) * 20, vg=rng.standard_normal((nlev, nlat, nlon)) * 20,
            psg=1e5 + 500 * rng.standard_normal((nlat, nlon)), dlnpsdt=1e-6 * rng.standard_normal((nlat, nlon)),
            gauwts=np.full(nlat, 2.0 / nlat))

def upload():
    d = {}
    for k, a in host.items():
        p = vp()
        assert rt.cudaMalloc(ctypes.byref(p), a.nbytes) == 0
        assert rt.cudaMemcpy(p, a.ctypes.data_as(vp), a.nbytes, H2D) == 0
        d[k] = p
    o = vp()
    assert rt.cudaMalloc(ctypes.byref(o), 32) == 0
    d["out"] = o
    return d

def call(d):
    rc = lib.gd_diag_static(d["ug"], d["vg"], nlev, d["psg"], d["dlnpsdt"], d["gauwts"], nlat, nlon, d["out"], None)
    assert rc == 0, rc
    out = np.zeros(4)
    assert rt.cudaMemcpy(out.ctypes.data_as(vp), d["out"], 32, D2H) == 0
    return out

a = call(upload())
assert rt.cudaDeviceReset() == 0  # ends this process's own context only
b = call(upload())
np.testing.assert_array_equal(a, b)
assert a[0] > 0
print("ok", a.tolist())
"""


def test_diag_static_after_device_reset(tmp_path):
    """A cudaDeviceReset in the caller's process ends its context and with it
    the device copy of the library's fixed scratch array; the next call, made
    under the new context, must find the array again rather than reuse the
    address it looked up under the old one.  Run in a child process that
    allocates its own inputs with cudaMalloc (it is the test harness, not a
    caller of the allocation-free path) and loads no other CUDA user."""
    import os
    import subprocess
    import sys

    env = dict(os.environ)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env["PYTHONPATH"] = os.pathsep.join([os.path.join(root, "gfs-dycore_gb300"), env.get("PYTHONPATH", "")])
    r = subprocess.run([sys.executable, "-c", _RESET_SCRIPT], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")

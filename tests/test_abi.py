"""CPU tests of the C-ABI boundary: the library builds, loads and exports
every entry point include/gd_api.h declares; argument validation returns
status codes without touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from gdpy import core, inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    hdr = open(os.path.join(ROOT, "include", "gd_api.h")).read()
    return set(re.findall(r"^\s*(?:int|const char\*|long long)\s+(gd_\w+)\s*\(", hdr, re.M))


def test_header_and_binding_agree():
    assert declared() == set(core.API_FUNCTIONS)


def test_library_exports_every_declared_symbol():
    lib = core.load()
    for name in declared():
        assert hasattr(lib, name), name


def test_default_config_matches_reference_namelist_defaults():
    c = core.default_config()
    # src/params.f90: massfix=.true., explicit=.false., ndiss=0, efold=0,
    # hdif_fac=hdif_fac2=1, fshk=0, taustratdamp=5 days
    assert c.massfix == 1 and c.explicit_ == 0 and c.ndiss == 0 and c.efold == 0
    assert c.hdif_fac == 1.0 and c.hdif_fac2 == 1.0 and c.fshk == 0
    assert c.taustratdamp == 5 * 86400.0


@pytest.mark.parametrize("kw,code", [
    (dict(nlon=100), core.GD_ERR_ARG),
    (dict(nlat=63), core.GD_ERR_ARG),
    (dict(ntrunc=64), core.GD_ERR_ARG),
    (dict(nlev=2), core.GD_ERR_ARG),
    (dict(dt=0.0), core.GD_ERR_ARG),
    (dict(precision=9), core.GD_ERR_ARG),
    (dict(dcmip=51, heldsuarez=1), core.GD_ERR_ARG),
    (dict(dcmip=30, heldsuarez=0), core.GD_ERR_ARG),
    (dict(dcmip=51, heldsuarez=0, dry=0, ntrac=0), core.GD_ERR_ARG),
])
def test_init_rejects_bad_config_without_gpu(kw, code):
    ak, bk = inputs.hybrid_coords(20)
    args = dict(ntrunc=42, nlon=128, nlat=64, nlev=20)
    args.update({k: kw.pop(k) for k in list(kw) if k in args})
    with pytest.raises(core.GdError) as e:
        core.Dycore(args["ntrunc"], args["nlon"], args["nlat"], args["nlev"], ak, bk, **kw)
    assert e.value.code == code


def test_null_arguments_are_rejected():
    lib = core.load()
    assert lib.gd_init(None, None, None, None) == core.GD_ERR_ARG
    assert lib.gd_finalize(None) == core.GD_ERR_ARG
    assert lib.gd_advance(None, ctypes.c_double(0.0), 1) == core.GD_ERR_ARG
    assert lib.gd_sync(None) == core.GD_ERR_ARG
    assert lib.gd_autotune(None, None) == core.GD_ERR_ARG
    assert lib.gd_set_closure(None, None) == core.GD_ERR_ARG
    assert lib.gd_closure_features(None, None) == core.GD_ERR_ARG
    assert lib.gd_ensemble_advance(None, 1, ctypes.c_double(0.0), 1) == core.GD_ERR_ARG
    for f in ("gd_mlp_destroy", "gd_mlp_sync"):
        assert getattr(lib, f)(None) == core.GD_ERR_ARG
    assert lib.gd_mlp_forward(None, None, 0, None) == core.GD_ERR_ARG
    assert lib.gd_mlp_train_step(None, None, None, 1, ctypes.c_float(1e-3), None) == core.GD_ERR_ARG
    assert lib.gd_mlp_init(4, 8, 1, 2, 0, 0, None) == core.GD_ERR_ARG
    # single-precision host entry points
    assert lib.gd_set_state_f(None, None, None, None, None, None, None) == core.GD_ERR_ARG
    assert lib.gd_get_state_f(None, None, None, None, None, None) == core.GD_ERR_ARG
    for f in ("gd_spectogrd_f", "gd_grdtospec_f"):
        assert getattr(lib, f)(None, 1, None, None) == core.GD_ERR_ARG
    assert lib.gd_getuv_f(None, 1, None, None, None, None) == core.GD_ERR_ARG
    assert lib.gd_getvrtdivspec_f(None, 1, None, None, None, None) == core.GD_ERR_ARG
    assert lib.gd_getgrad_f(None, 1, None, None, None) == core.GD_ERR_ARG
    assert lib.gd_get_topo(None, None) == core.GD_ERR_ARG


def test_hybrid_coordinate_is_valid():
    for L in (20, 64):
        ak, bk = inputs.hybrid_coords(L)
        assert ak[0] == 0 and bk[0] == 0 and bk[-1] == 1 and ak[-1] == 0
        p = ak + bk * 1e5
        assert np.all(np.diff(p) > 0) and np.all(ak >= 0)


def test_fortran_module_binds_every_declared_symbol():
    """include/gd_api.f90 has one bind(c) interface per entry point of
    include/gd_api.h (no Fortran compiler here: the check is textual)."""
    f90 = open(os.path.join(ROOT, "include", "gd_api.f90")).read()
    bound = set(re.findall(r"bind\(c, name='(gd_\w+)'\)", f90))
    assert bound == declared()


def test_shtns_module_has_the_reference_interface():
    """include/gd_shtns.f90 is module shtns with the public routines and
    module data of src/shtns.f90:58-60, each transform generic over the
    single- and double-precision kinds."""
    f90 = open(os.path.join(ROOT, "include", "gd_shtns.f90")).read()
    assert re.search(r"^module shtns$", f90, re.M)
    joined = re.sub(r"&\s*\n\s*", " ", f90)  # Fortran continuation lines
    public = set()
    for m in re.finditer(r"^\s*public ::(.*)$", joined, re.M):
        public |= {w.strip() for w in m.group(1).split(",") if w.strip()}
    assert public == {"shtns_init", "grdtospec", "spectogrd", "getuv", "getvrtdivspec", "getgrad",
                      "shtns_destroy", "gauwts", "lats", "lons", "nlm", "degree", "order", "lap", "invlap",
                      "current_nlon", "current_nlat", "current_ntrunc", "areawts"}
    for name in ("grdtospec", "spectogrd", "getuv", "getvrtdivspec", "getgrad"):
        assert re.search(rf"module procedure {name}_r4, {name}_r8", f90), name
        for k in ("r4", "r8"):
            assert re.search(rf"subroutine {name}_{k}\(", f90), (name, k)

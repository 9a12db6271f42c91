"""The C ABI: every entry point declared in include/*.h is exported by
libg3m3_gpu.so, the Python binding is derived from the header, and without
a GPU the library refuses to create a context instead of falling back."""
import ctypes
import os

import pytest

from _support import ROOT, has_gpu
from g3m3_gb300 import _lib


def test_header_lists_every_routine_of_the_path():
    names = {n for n, _, _ in _lib.header_functions()}
    for routine in ("push_ion", "push_elec", "push_bfld", "calcur", "fnd_evel", "fnd_vtot", "fnd_pres", "bande",
                    "lap_plasma", "lap_elec", "lap_bfld", "fcsmooth", "flux_correct", "set_rho", "set_speed_agrd",
                    "store_array", "bndry_outer", "bndry_inner", "flanks", "bndry_flanks", "corer", "bndry_corer",
                    "flanks_synced", "divb_correct", "sample_points"):
        assert "g3m3_" + routine in names, routine
    for fn in ("model_create", "model_run", "model_divb_all", "model_set_state", "model_get_state"):
        assert "g3m3_" + fn in names


def test_library_exports_every_declared_symbol():
    lib = _lib.load(build_if_missing=True)
    for name, ret, params in _lib.header_functions():
        fn = getattr(lib, name)
        assert fn.argtypes is not None and len(fn.argtypes) == len(params), name
    # drop-in signatures keep the reference's argument counts (+ the context)
    sig = {n: len(p) for n, _, p in _lib.header_functions()}
    assert sig["g3m3_push_ion"] == 1 + 62          # sub_push_ion.f90:4-17
    assert sig["g3m3_set_speed_agrd"] == 1 + 63    # sub_set_speed_agrd.f90:6-22
    assert sig["g3m3_bande"] == 1 + 38             # sub_BandE.f90:5-10
    assert sig["g3m3_lap_plasma"] == 1 + 33        # sub_lap_plasma.f90:4-10
    assert sig["g3m3_divb_correct"] == 1 + 13      # sub_divB_correct.f90:25-27 (+ iters)


def test_oracle_exports_its_header():
    from oracle import oracle
    L = oracle.lib()
    for name, _, params in _lib.header_functions(os.path.join(ROOT, "oracle", "g3m3_oracle.h"), "oracle_"):
        assert len(getattr(L, name).argtypes) == len(params)


@pytest.mark.skipif(has_gpu(), reason="checks the behaviour without a GPU")
def test_no_gpu_no_fallback():
    lib = _lib.load(build_if_missing=True)
    h = ctypes.c_void_p()
    assert lib.g3m3_ctx_create(ctypes.byref(h), 0) != 0
    from g3m3_gb300.api import Context, G3M3Error
    with pytest.raises(G3M3Error):
        Context(0)


def test_version_string():
    lib = _lib.load(build_if_missing=True)
    assert b"sm_103a" in lib.g3m3_version()

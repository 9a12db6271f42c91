"""The Fortran side of the drop-in (include/g3m3_stubs.f90), checked without
a Fortran compiler:

* the committed file is what include/make_fortran_stubs.py makes from
  include/g3m3.h today;
* every function of the header has an interface block with its C name, and
  every routine of the step has a stub;
* where the reference's sources are at hand ($G3M3_REFERENCE/code), every
  stub has the reference routine's name and its dummy list, name for name,
  so the main loop's calls bind to the stubs unchanged.
"""
import os
import re
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "include"))

import make_fortran_stubs as M  # noqa: E402

REF_FILES = {
    "push_ion": "sub_push_ion", "push_elec": "sub_push_elec", "push_bfld": "sub_push_bfld",
    "calcur": "sub_calcur", "fnd_evel": "sub_fnd_evel", "fnd_vtot": "sub_fnd_vtot", "BandE": "sub_BandE",
    "fnd_pres": "sub_fnd_pres", "lap_plasma": "sub_lap_plasma", "lap_elec": "sub_lap_elec",
    "lap_bfld": "sub_lap_bfld", "fcsmooth": "sub_fcsmooth", "set_rho": "sub_set_rho",
    "set_speed_agrd": "sub_set_speed_agrd", "store_array": "sub_store_array", "flanks": "sub_flanks",
    "corer": "sub_corer", "flanks_synced": "sub_flanks_synced", "divB_correct": "sub_divB_correct",
    "flux_counter": "sub_flux_counter", "sparse_solver": "sub_sparse_solver", "flux_correct": "sub_flux_correct",
    "bndry_outer": "sub_bndry_outer", "bndry_inner": "sub_bndry_inner", "bndry_flanks": "sub_bndry_flanks",
    "bndry_corer": "sub_bndry_corer",
}


def _text():
    return open(M.OUT).read()


def _stub_dummies(text):
    out = {}
    for m in re.finditer(r"^(?:recursive )?subroutine (\w+)\((.*?)\)\s*$", text, re.M | re.S):
        out[m.group(1)] = [a.strip() for a in re.sub(r"&\s*", "", m.group(2)).split(",")]
    return out


def test_stubs_file_is_current(tmp_path):
    _, text = M.generate(str(tmp_path / "g3m3_stubs.f90"))
    assert text == _text()


def test_every_header_function_and_routine_is_covered():
    text = _text()
    for name, _, _ in M.header_functions():
        assert f'bind(C, name="{name}")' in text, name
    stubs = _stub_dummies(text)
    assert set(REF_FILES) <= set(stubs), set(REF_FILES) - set(stubs)
    # the table routines pass every field of each table they build
    for ref, tables in (("flux_correct", ("", "wrk", "old")), ("bndry_flanks", ("wrk", "", "old")),
                        ("bndry_outer", ("",)), ("bndry_inner", ("",)), ("bndry_corer", ("",))):
        body = text[text.index(f"\nsubroutine {ref}("):text.index(f"end subroutine {ref}")]
        for pre in tables:
            for n in M.table_names(pre):
                assert f"c_loc({n}(1))" in body, (ref, n)
                assert f"real, target :: {n}(*)" in body, (ref, n)


def _reference_code():
    sys.path.insert(0, ROOT)
    import __graft_entry__
    code = os.path.join(__graft_entry__.REFERENCE, "code")
    return code if os.path.isdir(code) else None


@pytest.mark.skipif(_reference_code() is None, reason="reference sources absent")
def test_stub_dummies_are_the_reference_routines():
    code = _reference_code()
    stubs = _stub_dummies(_text())
    for ref, f in REF_FILES.items():
        src = open(os.path.join(code, f + ".f90")).read()
        m = re.search(r"^\s*(?:recursive\s+)?subroutine\s+(\w+)\s*\((.*?)\)", src, re.S | re.M | re.I)
        assert m.group(1) == ref, (f, m.group(1))
        args = re.sub(r"!.*", "", m.group(2))
        args = [a.strip().lower() for a in re.sub(r"[&\s]", "", args).split(",") if a.strip()]
        assert [a.lower() for a in stubs[ref]] == args, ref

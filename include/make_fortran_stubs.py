"""Writes include/g3m3_stubs.f90, the Fortran side of the drop-in boundary.

    python include/make_fortran_stubs.py

The file has three parts:

* module g3m3_c: a bind(C) derived type mirroring g3m3_params
  (include/g3m3_types.h) and one interface block per function of
  include/g3m3.h, generated from the header's prototypes (the parser of
  g3m3_gb300/_lib.py);
* module g3m3_stubs: the library context of the Fortran program, the status
  check (stop on error, warn on G3M3_ERR_NOCONV as the reference warns,
  sub_sparse_solver.f90:93,157) and the one-time initialisation;
* one external subroutine per reference routine on the step, with the
  reference's name and dummy list, forwarding to its g3m3_ entry: the main
  loop (code/3d_main.f90) calls them unchanged once they replace the
  sub_*.f90 files in the reference's makefile.  The five routines that
  pass all 34 fields (flux_correct, bndry_outer, bndry_inner, bndry_flanks,
  bndry_corer) build the library's pointer tables from their dummies, which
  carry the target attribute there (3d_main.f90 is not touched), and
  bndry_outer / bndry_inner fill a g3m3_params from their scalars and, for
  bndry_inner, the reference's common /rotation/ (v_rot).

No Fortran compiler exists in this build's images, so the file is not
compiled here; tests/test_fortran_stubs.py checks that it is current, that
it covers every header function and every routine, and (where the
reference's sources are at hand) that every stub's dummy list is the
reference routine's.
"""
from __future__ import annotations

import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "g3m3_stubs.f90")

SPECIES_FIELDS = ("rho", "px", "py", "pz", "presx", "presy", "presz", "presxy", "presxz", "presyz")


def table_names(prefix: str):
    """The 34 field names of a pointer table (g3m3_types.h order) with a
    name prefix ('', 'wrk', 'old') as the reference's dummies spell them."""
    out = [f"{prefix}{s}{f}" for s in "qho" for f in SPECIES_FIELDS]
    return out + [f"{prefix}epres", f"{prefix}bx", f"{prefix}by", f"{prefix}bz"]


# Reference routines forwarded one to one: reference name -> g3m3 entry.
DIRECT = {
    "push_ion": "g3m3_push_ion", "push_elec": "g3m3_push_elec", "push_bfld": "g3m3_push_bfld",
    "calcur": "g3m3_calcur", "fnd_evel": "g3m3_fnd_evel", "fnd_vtot": "g3m3_fnd_vtot",
    "BandE": "g3m3_bande", "fnd_pres": "g3m3_fnd_pres", "lap_plasma": "g3m3_lap_plasma",
    "lap_elec": "g3m3_lap_elec", "lap_bfld": "g3m3_lap_bfld", "fcsmooth": "g3m3_fcsmooth",
    "set_rho": "g3m3_set_rho", "set_speed_agrd": "g3m3_set_speed_agrd", "store_array": "g3m3_store_array",
    "flanks": "g3m3_flanks", "corer": "g3m3_corer", "flanks_synced": "g3m3_flanks_synced",
    "divB_correct": "g3m3_divb_correct", "flux_counter": "g3m3_flux_counter",
    "sparse_solver": "g3m3_sparse_solver",
}
# C arguments the reference routine does not have (filled by the stub)
EXTRA_OUT = {"divB_correct": {"iters"}}
RECURSIVE = {"sparse_solver"}
LOGICALS = {"isotropic", "recurse"}
# pointer arguments that are scalars on the Fortran side
SCALAR_OUT = {"pxmax", "pymax", "pzmax", "csmax", "alfmax", "fastest", "iters", "residual2", "qflux_in",
              "qflux_out", "hflux_in", "hflux_out", "oflux_in", "oflux_out", "loss", "t", "nsteps",
              "fcs_variant", "cell_updates", "kernels", "graphs", "ms_per_launch", "bytes"}

# The reference's dummy lists of the table routines (interfaces the main
# loop calls): sub_flux_correct.f90:4, sub_bndry_outer.f90:5,
# sub_bndry_inner.f90:5, sub_bndry_flanks.f90:5, sub_bndry_corer.f90:5.
_SP7 = ("rho", "presx", "presy", "presz", "px", "py", "pz")
_XYZ3 = ("presxy", "presxz", "presyz")


def _sp(prefix, s, names):
    return [f"{prefix}{s}{n}" for n in names]


FLUX_CORRECT = (
    sum(([*_sp("", s, ("rho", "presx", "presy", "presz", "presxy", "presxz", "presyz", "px", "py", "pz")),
          *_sp("wrk", s, ("rho", "presx", "presy", "presz", "presxy", "presxz", "presyz", "px", "py", "pz")),
          *_sp("old", s, ("rho", "presx", "presy", "presz", "presxy", "presxz", "presyz", "px", "py", "pz"))]
         for s in "qho"), [])
    + ["epres", "wrkepres", "oldepres", "bx", "by", "bz", "wrkbx", "wrkby", "wrkbz", "oldbx", "oldby", "oldbz",
       "vvx", "vvy", "vvz", "nx", "ny", "nz", "n_grids", "box", "difrho", "diferg", "xspac", "isotropic"])
BNDRY_OUTER = (
    sum((_sp("", s, _SP7) for s in "qho"), []) + ["epres"] + sum((_sp("", s, _XYZ3) for s in "qho"), [])
    + ["rmassq", "rmassh", "rmasso", "bx", "by", "bz", "bx0", "by0", "bz0", "nx", "ny", "nz", "n_grids",
       "srho", "rho_frac", "o_conc", "spress", "spx", "spy", "spz", "sbx_wind", "sby_wind", "sbz_wind",
       "ti_te", "isotropic"])
BNDRY_INNER = (
    sum((_sp("", s, _SP7) + [f"rmass{s}"] for s in "qho"), []) + ["epres", "bx", "by", "bz"]
    + sum((_sp("", s, _XYZ3) for s in "qho"), [])
    + ["nx", "ny", "nz", "n_grids", "parm_srf", "parm_mid", "parm_zero", "ijsrf", "numsrf", "ijmid", "nummid",
       "ijzero", "numzero", "mbndry", "msrf", "mmid", "mzero", "erho", "epress", "alpha_e", "ti_te", "o_conc",
       "re_equiv", "r_inner", "sbx_wind", "spress", "grd_xmin", "grd_xmax", "grd_ymin", "grd_ymax", "grd_zmin",
       "grd_zmax"])
_SP10 = ("rho", "px", "py", "pz", "presx", "presy", "presz", "presxy", "presxz", "presyz")
BNDRY_FLANKS = (
    sum((_sp("wrk", s, _SP10) for s in "qho"), []) + ["wrkepres", "wrkbx", "wrkby", "wrkbz"]
    + sum((_sp("", s, _SP10) for s in "qho"), []) + ["epres", "bx", "by", "bz"]
    + sum((_sp("old", s, _SP10) for s in "qho"), []) + ["oldepres", "oldbx", "oldby", "oldbz"]
    + ["work", "nx", "ny", "nz", "n_grids", "box", "t_old", "t_new", "t", "grd_xmin", "grd_xmax", "grd_ymin",
       "grd_ymax", "grd_zmin", "grd_zmax"])
BNDRY_CORER = (
    sum((_sp("", s, _SP7) for s in "qho"), []) + ["epres", "bx", "by", "bz"]
    + sum((_sp("", s, _XYZ3) for s in "qho"), [])
    + ["nx", "ny", "nz", "n_grids", "box", "grd_xmin", "grd_xmax", "grd_ymin", "grd_ymax", "grd_zmin",
       "grd_zmax"])
TABLE = {"flux_correct": FLUX_CORRECT, "bndry_outer": BNDRY_OUTER, "bndry_inner": BNDRY_INNER,
         "bndry_flanks": BNDRY_FLANKS, "bndry_corer": BNDRY_CORER}

_INTS = {"nx", "ny", "nz", "n_grids", "box", "mbndry", "msrf", "mmid", "mzero"}
_INT_ARRAYS = {"ijsrf", "numsrf", "ijmid", "nummid", "ijzero", "numzero"}
_DOUBLES = {"t_old", "t_new"}


def header_functions():
    sys.path.insert(0, ROOT)
    from g3m3_gb300 import _lib
    return _lib.header_functions()


def split_param(p):
    """(type, name, table_len) of one C parameter."""
    m = re.match(r"(.*?)(\w+)\s*(\[(\w+)\])?\s*$", p.strip())
    return m.group(1).strip(), m.group(2), m.group(4)


def wrap(head, items, tail="", indent="      "):
    """Fortran free-form lines of at most 100 characters."""
    lines, cur = [], head
    for k, it in enumerate(items):
        piece = it + (", " if k < len(items) - 1 else "")
        if len(cur) + len(piece) > 98:
            lines.append(cur.rstrip() + " &")
            cur = indent + piece
        else:
            cur += piece
    if len(cur) + len(tail) > 98:
        lines.append(cur.rstrip() + " &")
        cur = indent + tail.lstrip()
    else:
        cur += tail
    lines.append(cur)
    return lines


def f_decl(ctype, name, table):
    """The interface's declaration of one C parameter."""
    t = ctype.replace("const ", "").replace(" ", "")
    if table:
        return f"type(c_ptr) :: {name}(34)"
    if t in ("g3m3_ctx*", "g3m3_model*", "g3m3_ensemble*", "g3m3_adjoint*", "void*"):
        return f"type(c_ptr), value :: {name}"
    if t in ("g3m3_ctx**", "g3m3_model**", "g3m3_ensemble**", "g3m3_adjoint**"):
        return f"type(c_ptr), intent(out) :: {name}"
    if t == "g3m3_params*":
        return f"type(g3m3_params_t), intent(in) :: {name}"
    if t == "float*const*":
        return f"type(c_ptr) :: {name}(*)"
    if t == "char*":
        return f"character(kind=c_char) :: {name}(*)"
    base = {"float": "real(c_float)", "double": "real(c_double)", "int": "integer(c_int)",
            "size_t": "integer(c_size_t)", "unsignedlonglong": "integer(c_long_long)",
            "int64_t": "integer(c_int64_t)"}
    if t in base:
        return f"{base[t]}, value :: {name}"
    if t.endswith("*") and t[:-1] in base:
        b = base[t[:-1]]
        return f"{b} :: {name}" if name in SCALAR_OUT else f"{b} :: {name}(*)"
    raise ValueError(f"no Fortran form for {ctype} {name}")


def f_result(ret):
    r = ret.replace("const ", "").replace(" ", "")
    return {"int": "integer(c_int)", "size_t": "integer(c_size_t)", "char*": "type(c_ptr)",
            "void*": "type(c_ptr)"}[r]


def interfaces(funcs):
    L = ["  interface"]
    for name, ret, params in funcs:
        parts = [split_param(p) for p in params]
        names = [n for _, n, _ in parts]
        L += ["    " + x for x in wrap(f"function {name}(", names, f") bind(C, name=\"{name}\")")]
        L.append("      import")
        L.append(f"      {f_result(ret)} :: {name}")
        for t, n, tab in parts:
            L.append(f"      {f_decl(t, n, tab)}")
        L.append(f"    end function {name}")
    L.append("  end interface")
    return L


def params_type():
    sys.path.insert(0, ROOT)
    import ctypes
    from g3m3_gb300.params import G3M3Params
    L = ["  ! g3m3_params of include/g3m3_types.h, field for field", "  type, bind(C) :: g3m3_params_t"]
    for n, t in G3M3Params._fields_:
        if t is ctypes.c_int32:
            L.append(f"    integer(c_int32_t) :: {n} = 0")
        elif t is ctypes.c_float:
            L.append(f"    real(c_float) :: {n} = 0.")
        else:
            L.append(f"    real(c_float) :: {n}({t._length_}) = 0.")
    L.append("  end type g3m3_params_t")
    return L


def direct_stub(ref, cname, funcs):
    params = next(p for n, _, p in funcs if n == cname)
    parts = [split_param(p) for p in params[1:]]
    extra = EXTRA_OUT.get(ref, set())
    dummies = [n for _, n, _ in parts if n not in extra]
    L = []
    kw = "recursive subroutine" if ref in RECURSIVE else "subroutine"
    L += wrap(f"{kw} {ref}(", dummies, ")", indent="    ")
    L.append("  use g3m3_stubs")
    L.append("  implicit none")
    args = []
    for t, n, _ in parts:
        tt = t.replace("const ", "").replace(" ", "")
        base = {"float": "real", "double": "double precision", "int": "integer"}[tt.rstrip("*")]
        if n in extra:
            L.append(f"  {base} :: {n}")
            args.append(n)
        elif n in LOGICALS:
            L.append(f"  logical :: {n}")
            args.append(f"merge(1_c_int, 0_c_int, {n})")
        elif tt.endswith("*") and n not in SCALAR_OUT:
            L.append(f"  {base} :: {n}(*)")
            args.append(n)
        else:
            L.append(f"  {base} :: {n}")
            args.append(n)
    L.append("  call g3m3_init(0)")
    L += wrap(f"  call g3m3_check({cname}(g3m3_ctx, ", args, f"), '{ref}')", indent="      ")
    L.append(f"end subroutine {ref}")
    return L


def table_stub(ref, dummies):
    tables = {"flux_correct": [("cur", ""), ("wrk", "wrk"), ("old", "old")],
              "bndry_outer": [("f", "")], "bndry_inner": [("f", "")],
              "bndry_flanks": [("tgt", "wrk"), ("cur", ""), ("old", "old")], "bndry_corer": [("f", "")]}[ref]
    fields = set()
    for _, pre in tables:
        fields |= set(table_names(pre))
    L = wrap(f"subroutine {ref}(", dummies, ")", indent="    ")
    L.append("  use g3m3_stubs")
    L.append("  implicit none")
    for n in dummies:
        if n in fields:
            L.append(f"  real, target :: {n}(*)")
        elif n in LOGICALS:
            L.append(f"  logical :: {n}")
        elif n in _INTS:
            L.append(f"  integer :: {n}")
        elif n in _INT_ARRAYS:
            L.append(f"  integer :: {n}(*)")
        elif n in _DOUBLES:
            L.append(f"  double precision :: {n}(*)")
        elif n == "t":
            L.append(f"  double precision :: {n}")
        elif n in ("vvx", "vvy", "vvz", "xspac", "work", "bx0", "by0", "bz0", "parm_srf", "parm_mid",
                   "parm_zero") or n.startswith("grd_"):
            L.append(f"  real :: {n}(*)")
        else:
            L.append(f"  real :: {n}")
    for tab, _ in tables:
        L.append(f"  type(c_ptr) :: {tab}(34)")
    if ref in ("bndry_outer", "bndry_inner"):
        L.append("  type(g3m3_params_t) :: p   ! every component starts at zero")
    if ref == "bndry_inner":
        L.append("  real :: v_rot, r_rot, rot_angle, xdip, ydip, zdip, sin_tilt, cos_tilt, b0")
        L.append("  common /rotation/ v_rot, r_rot, rot_angle, xdip, ydip, zdip, sin_tilt, cos_tilt, b0")
    for tab, pre in tables:
        for k, n in enumerate(table_names(pre)):
            L.append(f"  {tab}({k + 1}) = c_loc({n}(1))")
    if ref in ("bndry_outer", "bndry_inner"):
        L += ["  p%nx = nx", "  p%ny = ny", "  p%nz = nz", "  p%n_grids = n_grids",
              "  p%rmassq = rmassq", "  p%rmassh = rmassh", "  p%rmasso = rmasso",
              "  p%o_conc = o_conc", "  p%ti_te = ti_te", "  p%spress = spress", "  p%sbx_wind = sbx_wind"]
    if ref == "bndry_outer":
        L += ["  p%isotropic = merge(1, 0, isotropic)", "  p%srho = srho", "  p%rho_frac = rho_frac",
              "  p%spx = spx", "  p%spy = spy", "  p%spz = spz", "  p%sby_wind = sby_wind",
              "  p%sbz_wind = sbz_wind"]
        call = ["g3m3_ctx", "f", "bx0", "by0", "bz0", "p"]
    elif ref == "bndry_inner":
        L += ["  p%mbndry = mbndry", "  p%erho = erho", "  p%epress = epress", "  p%alpha_e = alpha_e",
              "  p%re_equiv = re_equiv", "  p%r_inner = r_inner", "  p%v_rot = v_rot",
              "  p%grd_xmin(1:n_grids) = grd_xmin(1:n_grids)", "  p%grd_xmax(1:n_grids) = grd_xmax(1:n_grids)",
              "  p%grd_ymin(1:n_grids) = grd_ymin(1:n_grids)", "  p%grd_ymax(1:n_grids) = grd_ymax(1:n_grids)",
              "  p%grd_zmin(1:n_grids) = grd_zmin(1:n_grids)", "  p%grd_zmax(1:n_grids) = grd_zmax(1:n_grids)"]
        call = ["g3m3_ctx", "f", "parm_srf", "parm_mid", "parm_zero", "ijsrf", "numsrf", "ijmid", "nummid",
                "ijzero", "numzero", "msrf", "mmid", "mzero", "p"]
    elif ref == "flux_correct":
        call = ["g3m3_ctx", "cur", "wrk", "old", "nx", "ny", "nz", "n_grids", "box", "difrho", "diferg"]
    elif ref == "bndry_flanks":
        call = ["g3m3_ctx", "tgt", "cur", "old", "nx", "ny", "nz", "n_grids", "box", "t_old", "t_new", "t",
                "grd_xmin", "grd_xmax", "grd_ymin", "grd_ymax", "grd_zmin", "grd_zmax"]
    else:
        call = ["g3m3_ctx", "f", "nx", "ny", "nz", "n_grids", "box", "grd_xmin", "grd_xmax", "grd_ymin",
                "grd_ymax", "grd_zmin", "grd_zmax"]
    L.append("  call g3m3_init(0)")
    L += wrap(f"  call g3m3_check(g3m3_{ref}(", call, f"), '{ref}')", indent="      ")
    L.append(f"end subroutine {ref}")
    return L


STUBS_MODULE = """\
module g3m3_stubs
  use iso_c_binding
  use g3m3_c
  implicit none
  type(c_ptr), save :: g3m3_ctx = c_null_ptr
contains
  ! stop with the library's message on an error; G3M3_ERR_NOCONV (3) is
  ! the solver's "too many iterations", a warning in the reference
  subroutine g3m3_check(rc, what)
    integer(c_int), intent(in) :: rc
    character(*), intent(in) :: what
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (rc == 0) return
    call c_f_pointer(g3m3_last_error(g3m3_ctx), msg, [512])
    n = 0
    do while (n < 512)
      if (msg(n + 1) == c_null_char) exit
      n = n + 1
    end do
    write(*, *) 'g3m3: ', what, ': ', msg(1:n)
    if (rc /= 3) stop
  end subroutine g3m3_check

  subroutine g3m3_init(device)
    integer, intent(in) :: device
    if (c_associated(g3m3_ctx)) return
    if (g3m3_ctx_create(g3m3_ctx, int(device, c_int)) /= 0) stop 'g3m3: no GPU context'
  end subroutine g3m3_init
end module g3m3_stubs
"""


def generate(path=OUT):
    funcs = header_functions()
    L = ["! g3m3_stubs.f90 -- GENERATED by include/make_fortran_stubs.py from include/g3m3.h;",
         "! do not edit.  Not compiled in this build (no Fortran compiler in its images).",
         "!",
         "! The Fortran side of the drop-in: replace the reference's sub_*.f90 files of",
         "! the routines below by this file in its makefile and link",
         "! -L<repo>/g3m3_gb300/lib -lg3m3_gpu.  Default REAL and INTEGER must be",
         "! 4 bytes (c_float, c_int), as the reference builds them.",
         "",
         "module g3m3_c",
         "  use iso_c_binding",
         "  implicit none"]
    L += params_type()
    L += interfaces(funcs)
    L.append("end module g3m3_c")
    L.append("")
    L += STUBS_MODULE.splitlines()
    for ref, cname in DIRECT.items():
        L.append("")
        L += direct_stub(ref, cname, funcs)
    for ref, dummies in TABLE.items():
        L.append("")
        L += table_stub(ref, dummies)
    text = "\n".join(L) + "\n"
    old = open(path).read() if os.path.exists(path) else None
    if text != old:
        with open(path, "w") as fh:
            fh.write(text)
    return path, text


if __name__ == "__main__":
    print(generate()[0])

"""ctypes mirror of ``g3m3_params`` (include/g3m3_types.h) and field tables.

The reference keeps these constants in Fortran namelists, compile-time
parameters and common blocks (code/3d_main.f90:54-163, 582-602); here they
are one plain-C struct shared by the GB300 library and its callers.
"""
import ctypes

MAX_GRIDS = 16
NFIELDS = 34

# Field order of every table (fluid-file record order, 3d_main.f90:3310-3349).
SPECIES = ("q", "h", "o")
SPECIES_FIELDS = ("rho", "px", "py", "pz", "presx", "presy", "presz",
                  "presxy", "presxz", "presyz")
FIELD_NAMES = tuple(f"{s}{f}" for s in SPECIES for f in SPECIES_FIELDS) + (
    "epres", "bx", "by", "bz")
F = {name: i for i, name in enumerate(FIELD_NAMES)}
F_EPRES, F_BX, F_BY, F_BZ = 30, 31, 32, 33

_FLOAT_FIELDS = (
    "rmassq rmassh rmasso gamma gamma1 reynolds resist grav re_equiv "
    "chirho chipxyz chierg difrho diferg smallbit aniso_limit vlim_factor "
    "qvlim hvlim ovlim qclim hclim oclim cslim stepsz t_step_max t_step_min "
    "srho rho_frac o_conc spress spx spy spz sbx_wind sby_wind sbz_wind ti_te "
    "erho epress alpha_e r_inner v_rot r_rot divb_errlim pad1").split()


class G3M3Params(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_int32) for n in
                 ("nx", "ny", "nz", "n_grids", "mbndry", "isotropic",
                  "divb_every", "pad0")]
                + [(n, ctypes.c_float * MAX_GRIDS) for n in
                   ("xspac", "grd_xmin", "grd_xmax", "grd_ymin", "grd_ymax",
                    "grd_zmin", "grd_zmax")]
                + [(n, ctypes.c_float) for n in _FLOAT_FIELDS])

    def box_cells(self):
        return self.nx * self.ny * self.nz

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v)[: self.n_grids] if hasattr(v, "__len__") else v
        return out

"""``torch.ops.g3m3``: the drop-in routines of include/g3m3.h as PyTorch
operators on CUDA tensors.

Every routine of the step's C ABI (the reference subroutines, argument for
argument, minus the context) is registered as ``torch.ops.g3m3.<routine>``,
its schema read from the header:

* a REAL array is a contiguous float32 CUDA tensor; the reference's
  ``A(nx,ny,nz,n_grids)`` is a tensor of shape (n_grids, nz, ny, nx);
* a 34-field table (``float* const f[G3M3_NFIELDS]``) is a list of 34 such
  tensors, in the field order of include/g3m3_types.h;
* INTEGER arrays (the inner-boundary lists, the band layout) are int32
  tensors, real(dp) times float64 tensors, the parameter block of
  bndry_outer/bndry_inner a uint8 tensor (:func:`params_tensor`);
* scalars are Python numbers.

The arrays a routine writes are declared mutated (``Tensor(a!)``).  The
results the reference returns through scalar dummies (set_speed_agrd's
six maxima, divB_correct's iteration count, sparse_solver's residual,
flux_counter's six wall fluxes) are the op's return values.

The ops run on one library context per device, on its stream, ordered
after the work already queued on torch's current stream and before the
work queued on it afterwards.  Importing this module registers the ops.
"""
from __future__ import annotations

import ctypes
import re

import torch

from . import _lib
from .api import Context, table

# routines registered (the drop-in entries and the sampling helper)
ROUTINES = (
    "push_ion", "push_elec", "push_bfld", "calcur", "total_b", "fnd_evel", "fnd_vtot", "bande", "fnd_pres",
    "lap_plasma", "lap_elec", "lap_bfld", "fcsmooth", "flux_correct", "set_rho", "set_speed_agrd",
    "store_array", "bndry_outer", "bndry_inner", "flanks", "bndry_flanks", "corer", "bndry_corer",
    "flanks_synced", "divb_correct", "divb_correct_noalloc", "flux_counter", "sparse_solver", "sample_points",
)

# pointer dummies that carry a scalar result, not an array
SCALAR_RESULTS = {
    "set_speed_agrd": ("pxmax", "pymax", "pzmax", "csmax", "alfmax", "fastest"),
    "divb_correct": ("iters",),
    "divb_correct_noalloc": ("iters",),
    "sparse_solver": ("residual2",),
    "flux_counter": ("qflux_in", "qflux_out", "hflux_in", "hflux_out", "oflux_in", "oflux_out"),
}


def _param(p: str):
    """(kind, name) of one C parameter: kind is 'array' (written), 'in'
    (read), 'table' (written table), 'intable' (read table), 'params',
    'int', 'float' or 'double'."""
    name = re.sub(r"\[.*\]", "", p.split()[-1]).lstrip("*")
    body = " ".join(p.split()[:-1])
    is_table = "[" in p
    if "g3m3_params" in body:
        return "params", name
    if "*" in body or is_table:
        const_data = body.startswith("const")
        if is_table:
            return ("intable" if const_data else "table"), name
        return ("in" if const_data else "array"), name
    return body.split()[-1], name


def signature(routine: str):
    """[(kind, name)] of g3m3_<routine>'s parameters after the context,
    scalar results marked 'result_float' / 'result_int'."""
    for fname, _, params in _lib.header_functions():
        if fname == "g3m3_" + routine:
            out = []
            for p in params[1:]:
                kind, name = _param(p)
                if name in SCALAR_RESULTS.get(routine, ()):
                    kind = "result_int" if p.replace(" ", "").startswith("int*") else "result_float"
                out.append((kind, name))
            return out
    raise KeyError(routine)


def schema(routine: str) -> str:
    args, rets, k = [], [], 0
    for kind, name in signature(routine):
        arg = name + "_" if name in ("out", "self") else name
        if kind == "array":
            args.append(f"Tensor(a{k}!) {arg}")
            k += 1
        elif kind == "table":
            args.append(f"Tensor(a{k}!)[] {arg}")
            k += 1
        elif kind == "intable":
            args.append(f"Tensor[] {arg}")
        elif kind in ("in", "params"):
            args.append(f"Tensor {arg}")
        elif kind == "int":
            args.append(f"int {arg}")
        elif kind in ("float", "double"):
            args.append(f"float {arg}")
        elif kind == "result_float":
            rets.append("float")
        elif kind == "result_int":
            rets.append("int")
        else:
            raise ValueError(f"{routine}: parameter kind {kind}")
    ret = "()" if not rets else (rets[0] if len(rets) == 1 else "(" + ", ".join(rets) + ")")
    return f"{routine}({', '.join(args)}) -> {ret}"


_CONTEXTS = {}


def context(device: int) -> Context:
    """The library context the ops use on ``device``."""
    if device not in _CONTEXTS:
        _CONTEXTS[device] = Context(device)
    return _CONTEXTS[device]


def params_tensor(p) -> torch.Tensor:
    """The bytes of a g3m3_params block (g3m3_gb300.params.G3M3Params) as a
    CPU uint8 tensor, the form bndry_outer and bndry_inner take."""
    return torch.frombuffer(bytearray(bytes(p)), dtype=torch.uint8).clone()


def _tensor_addr(t: torch.Tensor, routine: str, name: str):
    if not t.is_contiguous():
        raise ValueError(f"g3m3.{routine}: {name} must be contiguous")
    return t.data_ptr()


def _implementation(routine: str):
    sig = signature(routine)

    def run(*args):
        device = next(a.device for a in _flat_tensors(args) if a.is_cuda)
        ctx = context(device.index if device.index is not None else torch.cuda.current_device())
        conv, results = [], []
        it = iter(args)
        for kind, name in sig:
            if kind in ("result_float", "result_int"):
                r = ctypes.c_int() if kind == "result_int" else ctypes.c_float()
                results.append(r)
                conv.append(ctypes.addressof(r))
                continue
            a = next(it)
            if kind in ("array", "in", "params"):
                conv.append(_tensor_addr(a, routine, name))
            elif kind in ("table", "intable"):
                conv.append(table([_tensor_addr(t, routine, name) for t in a]))
            else:
                conv.append(a)
        torch_stream = torch.cuda.current_stream(device)
        lib_stream = torch.cuda.ExternalStream(ctx.L.g3m3_ctx_stream(ctx.h), device=device)
        lib_stream.wait_stream(torch_stream)
        ctx.call(routine, *conv)
        torch_stream.wait_stream(lib_stream)
        vals = [r.value for r in results]
        if not vals:
            return None
        return vals[0] if len(vals) == 1 else tuple(vals)

    return run


def _flat_tensors(args):
    for a in args:
        if isinstance(a, torch.Tensor):
            yield a
        elif isinstance(a, (list, tuple)):
            yield from (t for t in a if isinstance(t, torch.Tensor))


_LIB = None


def register():
    """Define torch.ops.g3m3.* (once per process)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    lib = torch.library.Library("g3m3", "DEF")
    for r in ROUTINES:
        lib.define(schema(r))
        lib.impl(r, _implementation(r), "CUDA")
    _LIB = lib
    return lib


register()

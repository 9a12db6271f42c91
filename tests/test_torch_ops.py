"""torch.ops.g3m3 (g3m3_gb300/torch_ops.py), without a GPU: every drop-in
routine of the step is registered, and each schema declares mutated exactly
the arrays the C ABI takes as writable (non-const pointers), with the
scalar results as return values."""
import re
import sys
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "include"))

torch = pytest.importorskip("torch")


def test_every_step_routine_is_an_op():
    import g3m3_gb300.torch_ops as T
    from test_fortran_stubs import REF_FILES
    for ref in REF_FILES:
        r = ref.lower()
        assert r in T.ROUTINES, r
        assert hasattr(torch.ops.g3m3, r), r


def test_schemas_follow_the_header():
    import g3m3_gb300.torch_ops as T
    from g3m3_gb300 import _lib
    params = {n[len("g3m3_"):]: p for n, _, p in _lib.header_functions()}
    for r in T.ROUTINES:
        op = getattr(torch.ops.g3m3, r).default
        args = op._schema.arguments
        mutated = {a.name.rstrip("_") for a in args if a.alias_info is not None and a.alias_info.is_write}
        results = set(T.SCALAR_RESULTS.get(r, ()))
        writable = set()
        for p in params[r][1:]:
            name = re.sub(r"\[.*\]", "", p.split()[-1]).lstrip("*")
            body = " ".join(p.split()[:-1])
            if ("*" in body or "[" in p) and not body.startswith("const") and "g3m3_params" not in body:
                writable.add(name)
        assert mutated == writable - results, (r, mutated ^ (writable - results))
        assert len(args) == len(params[r]) - 1 - len(results), r
        assert len(op._schema.returns) == len(results), r

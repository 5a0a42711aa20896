"""The C-ABI library loads without a GPU and exports every declared symbol;
host-only entry points (falloff tables, argument checks) agree with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from dune_sculpt_gb300 import build as libbuild
from dune_sculpt_gb300 import sculpt, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    libbuild.build()
    return sculpt.load()


def declared_symbols():
    out = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            out |= set(re.findall(r"\b(sgpu_[a-z0-9_]+)\s*\(", text))
    return out


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 25
    for s in sorted(syms):
        assert hasattr(lib, s), f"{s} declared in include/ but not exported"
    assert set(sculpt.EXPORTS) <= syms


def test_curve_table_matches_oracle(lib, oracle):
    for preset in (0, 1, 2, 3, 5, 6):
        t_gpu, p_gpu = sculpt.curve_table(preset)
        t_or, p_or = oracle.curve_table(preset)
        assert np.array_equal(t_gpu.view(np.uint32), t_or.view(np.uint32)), preset
        assert np.array_equal(p_gpu.view(np.uint32), p_or.view(np.uint32)), preset


def test_invalid_arguments_return_codes(lib):
    with pytest.raises(sculpt.SculptGPUError) as e:
        sculpt.curve_table(42)
    assert e.value.code == sculpt.ERR_INVALID_ARG
    h = C.c_void_p()
    rc = lib.sgpu_mesh_create_faces(None, 0, None, 0, None, 0, None, 0, None, None, None, 0,
                                    C.byref(h))
    assert rc == sculpt.ERR_INVALID_ARG
    assert lib.sgpu_mesh_destroy(None) == sculpt.ERR_INVALID_ARG
    assert lib.sgpu_pbvh_update_normals(None) == sculpt.ERR_INVALID_ARG
    assert b"NULL" in lib.sgpu_last_error()


def test_version(lib):
    assert b"sm_103a" in lib.sgpu_version()


def test_debug_inject_arguments(lib):
    """The failure-injection hooks are host-side switches: they take and
    reject values without touching a device."""
    assert lib.sgpu_debug_inject(99, 0) == sculpt.ERR_INVALID_ARG
    assert lib.sgpu_debug_inject(sculpt.INJECT_ALLOC_FAIL, -1) == sculpt.ERR_INVALID_ARG
    assert lib.sgpu_debug_inject(sculpt.INJECT_BARRIER_EXTRA, 2) == sculpt.ERR_INVALID_ARG
    for what, value in ((sculpt.INJECT_ALLOC_FAIL, 3), (sculpt.INJECT_WAIT_NS, 1000),
                        (sculpt.INJECT_BARRIER_EXTRA, 1)):
        assert lib.sgpu_debug_inject(what, value) == sculpt.OK
    for what in (sculpt.INJECT_ALLOC_FAIL, sculpt.INJECT_WAIT_NS, sculpt.INJECT_BARRIER_EXTRA):
        assert lib.sgpu_debug_inject(what, 0) == sculpt.OK

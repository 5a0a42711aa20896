"""A compiled C caller of the C ABI (tests/c_abi/dab_sequence.c, C99, with
static checks that the element structs have the reference's layouts): it
builds and links here; on a GPU it runs the per-dab sequence a reference-side
stroke makes (search, do_draw_brush per symmetry pass, normal update, bounds
refit) and its positions, normals and node boxes equal the oracle's stroke bit
for bit."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from dune_sculpt_gb300 import build as libbuild
from dune_sculpt_gb300 import synth

from helpers import bits_equal, small_icosphere

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_abi", "dab_sequence.c")


def compile_caller(outdir: str) -> str:
    lib = libbuild.build()
    exe = os.path.join(outdir, "dab_sequence")
    cmd = [shutil.which("gcc") or "gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
           "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", os.path.dirname(lib), "-lsculptgpu", "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_caller_compiles_and_links():
    with tempfile.TemporaryDirectory() as d:
        exe = compile_caller(d)
        assert os.path.exists(exe)


@pytest.mark.gpu
@pytest.mark.parametrize("symmetry", [0, synth.SYMM_X])
def test_c_caller_matches_oracle(gpu, oracle, symmetry):
    m = small_icosphere(5, masked=False)  # the C caller passes no mask
    ll = 600
    st = synth.Stroke(synth.TOOL_DRAW, 0.15, 0.5, synth.CURVE_SMOOTH, symmetry,
                      synth.arc_dabs(11, 16, 0.04))
    with tempfile.TemporaryDirectory() as d:
        exe = compile_caller(d)
        mesh_bin, dabs_bin, out_bin = (os.path.join(d, n) for n in ("m.bin", "d.bin", "o.bin"))
        with open(mesh_bin, "wb") as f:
            np.array([m.verts.shape[0], m.polys.shape[0], m.loops.shape[0],
                      m.looptris.shape[0], ll], np.int32).tofile(f)
            for a in (m.verts, m.polys, m.loops, m.looptris):
                np.ascontiguousarray(a).tofile(f)
        with open(dabs_bin, "wb") as f:
            np.array([st.dabs.shape[0], symmetry], np.int32).tofile(f)
            np.array([st.radius, st.strength], np.float32).tofile(f)
            np.ascontiguousarray(st.dabs, dtype=np.float32).tofile(f)
        r = subprocess.run([exe, mesh_bin, dabs_bin, out_bin], capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr
        raw = np.fromfile(out_bin, dtype=np.uint8)
    V = m.verts.shape[0]
    o = oracle.OracleMesh.faces(m, ll)
    o.recalc_all_normals()
    tot, _ = o.stroke(st, which=1)
    assert tot > 0
    N = o.num_nodes
    verts = raw[:16 * V].view(synth.MVERT_DT)
    no = raw[16 * V:28 * V].view(np.float32).reshape(V, 3)
    boxes = raw[28 * V:].view(np.float32)
    assert boxes.size == 12 * N
    vb, ovb = boxes[:6 * N].reshape(N, 6), boxes[6 * N:].reshape(N, 6)
    co = np.ascontiguousarray(verts["co"])
    assert bits_equal(co, o.co())
    assert bits_equal(no, o.no())
    ob_vb, ob_ovb = o.bbs()
    assert bits_equal(vb, ob_vb) and bits_equal(ovb, ob_ovb)

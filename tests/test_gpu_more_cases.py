"""More parity cases of the GPU path against the oracle (bit for bit, plus the
FP64 bound): n-gon polygons (Newell normals, fan looptris), meshes whose
leaves split by material, all three mirror axes (seven passes per dab), every
falloff preset, smooth strengths on the sweep-count boundaries, clay strips
with a plane offset and other area / normal radius factors."""
import numpy as np
import pytest

from dune_sculpt_gb300 import synth
from dune_sculpt_gb300.sculpt import PBVH, STROKE_EAGER, STROKE_GRAPH, STROKE_TEAM

from helpers import bits_equal, first_diff, material_grid, ngon_mesh, rel_err, small_icosphere

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-6
FP64_TOL_PINCHING = 2e-6  # pinch / crease: FP32 drift of the centre pull (GPU = FP32 exactly)
TOOLS = (synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_INFLATE, synth.TOOL_CLAY_STRIPS,
         synth.TOOL_PINCH, synth.TOOL_CREASE)


def _pair(oracle, m, ll):
    g = PBVH.build_mesh(m, ll)
    o = oracle.OracleMesh.faces(m, ll)
    o.recalc_all_normals()
    return g, o


def _check(g, o, st, mode, tools=None, what=""):
    s = g.stroke(st, mode=mode, dab_tools=tools)
    tot, _ = o.stroke(st, which=3, dab_tools=tools)
    assert s.verts_displaced == tot, what
    assert bits_equal(g.positions(), o.co()), what + " co " + first_diff(g.positions(), o.co())
    assert bits_equal(g.normals(), o.no()), what + " no " + first_diff(g.normals(), o.no())
    for a, b in zip(g.bbs(), o.bbs()):
        assert bits_equal(a, b), what + " bb " + first_diff(a, b)
    pinching = (st.tool in (synth.TOOL_PINCH, synth.TOOL_CREASE) or
                (tools is not None and np.isin(tools, (synth.TOOL_PINCH, synth.TOOL_CREASE)).any()))
    assert rel_err(g.positions(), o.co64()) < (FP64_TOL_PINCHING if pinching else FP64_TOL), what
    return tot


@pytest.mark.parametrize("tool", TOOLS)
@pytest.mark.parametrize("mode", [STROKE_GRAPH, STROKE_TEAM])
def test_ngon_mesh_strokes(gpu, oracle, tool, mode):
    m = ngon_mesh(60)
    g, o = _pair(oracle, m, 400)
    st = synth.Stroke(tool, 0.12, 0.7, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.line_dabs(synth.SEED_BASE + 3, 16))
    assert _check(g, o, st, mode, what=f"ngon tool {tool}") > 0


@pytest.mark.parametrize("mode", [STROKE_GRAPH, STROKE_TEAM])
def test_material_split_mesh(gpu, oracle, mode):
    m = material_grid(64)
    g, o = _pair(oracle, m, 500)
    tools = np.array([TOOLS[d % len(TOOLS)] for d in range(20)], dtype=np.int32)
    st = synth.Stroke(synth.TOOL_DRAW, 0.1, 0.6, synth.CURVE_SMOOTH, 0,
                      synth.line_dabs(synth.SEED_BASE + 4, 20))
    assert _check(g, o, st, mode, tools, "materials") > 0


@pytest.mark.parametrize("tool", [synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_CLAY_STRIPS])
@pytest.mark.parametrize("mode", [STROKE_EAGER, STROKE_TEAM])
def test_xyz_symmetry(gpu, oracle, tool, mode):
    m = small_icosphere(4)
    g, o = _pair(oracle, m, 200)
    st = synth.Stroke(tool, 0.15, 0.6, synth.CURVE_SMOOTH, 7, synth.arc_dabs(19, 12, 0.05))
    assert _check(g, o, st, mode, what=f"xyz tool {tool}") > 0


@pytest.mark.parametrize("preset", [0, 1, 2, 3, 5, 6])
def test_falloff_presets(gpu, oracle, preset):
    m = small_icosphere(4)
    g, o = _pair(oracle, m, 200)
    st = synth.Stroke(synth.TOOL_INFLATE, 0.2, 0.5, preset, synth.SYMM_X,
                      synth.arc_dabs(23, 10, 0.05))
    assert _check(g, o, st, STROKE_TEAM, what=f"preset {preset}") > 0


@pytest.mark.parametrize("strength", [0.25, 0.5, 0.999, 1.0, 1.5])
def test_smooth_sweep_boundaries(gpu, oracle, strength):
    """Strengths at count = (int)(4 s) boundaries: the last sweep's strength
    4 (s - count / 4) is 0 at 0.25, 0.5 and 1.0; 1.5 clamps to 1."""
    m = small_icosphere(4)
    g, o = _pair(oracle, m, 200)
    st = synth.Stroke(synth.TOOL_SMOOTH, 0.2, strength, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.arc_dabs(29, 10, 0.05))
    _check(g, o, st, STROKE_TEAM, what=f"strength {strength}")


def test_clay_strips_plane_offset_and_factors(gpu, oracle):
    m = small_icosphere(4)
    g, o = _pair(oracle, m, 200)
    st = synth.Stroke(synth.TOOL_CLAY_STRIPS, 0.2, 0.8, synth.CURVE_SHARP, synth.SYMM_X,
                      synth.arc_dabs(31, 12, 0.05), normal_radius_factor=0.3,
                      area_radius_factor=0.8, plane_offset=0.2)
    assert _check(g, o, st, STROKE_TEAM, what="clay offset") > 0


def test_area_normal_center_matches_oracle(gpu, oracle):
    """sgpu_calc_area_normal_and_center: bit-equal to the FP32 restatement and
    within 1e-6 of an FP64 reduction of the same vertex set, FACES and GRIDS."""
    from helpers import small_uvsphere

    m = small_uvsphere(128)
    cases = [(PBVH.build_mesh(m, 800), oracle.OracleMesh.faces(m, 800), synth.arc_dabs(7, 20, 0.05))]
    gr = synth.torus_grids(16, 6, level=4)
    cases.append((PBVH.build_grids(gr, 4), oracle.OracleMesh.grids(gr, 4), synth.torus_dabs(9, 20, 0.1)))
    st = synth.Stroke(synth.TOOL_CLAY_STRIPS, 0.12, 0.8, synth.CURVE_SHARP, 0, None)
    for g, o, dabs in cases:
        o.recalc_all_normals()
        for d in range(dabs.shape[0]):
            loc = dabs[d, :3]
            nodes = o.search_sphere(loc, float(np.float32(np.float32(0.12) * np.float32(0.12))))
            a32, a64 = o.area_normal_center(st, loc, nodes)
            no, co = g.area_normal_center(st, loc, nodes)
            assert np.array_equal(np.concatenate([no, co]).view(np.uint32), a32.view(np.uint32)), d
            assert np.abs(a32.astype(np.float64) - a64).max() <= 1e-6, d

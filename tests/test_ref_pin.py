"""The oracle pinned to the reference's own code, compiled here.

oracle/Makefile target `ref` compiles, from the reference checkout, the
shaderio headers (shaders/shaderio*.h) as C++ and the shader functions of
shaders/tessellation.glsl:28-201, culling.glsl:27-92 and displacement.glsl:27-120
through a syntax-only rewrite (oracle/glsl_to_cpp.py) over a GLSL built-in shim
(oracle/ref_shim/glsl_shim.h), next to the oracle. Compiling checks every
field of 16 structs of include/tc_tessellation.h against the reference's
layout; running compares each reference function with the oracle's restatement
on exhaustive and seeded inputs. Skipped where the reference checkout is absent
(oracle/Makefile says where it looks)."""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PIN = os.path.join(ROOT, "oracle", "_ref", "ref_shader_pin")

# check -> least number of inputs compared at the default sample scale
COVERAGE = {
    "tess_encodeBarycentrics": 4_000_000,
    # every encoding of a point of the triangle (u + v <= 32768) plus 16 M random words
    "tess_decodeBarycentrics": 32769 * 32770 // 2 + 16_000_000,
    "tess_getTessFactors": 2_000_000,
    "tess_getSplitFactor": 10 * 32768,  # split factors 2..11, every factor 1..32768
    "tess_getConfig": 15 ** 3 * 6,  # every factor triple of the lookup, six vertex orders
    "tess_getConfigTriangleVertices": 2 * 14832,  # every table triangle of every config, both windings
    "tess_getConfigVertexBarycentrics": 2 * 12531,
    "tess_getConfigTriangleCount/VertexCount": 1012,
    "tess_interpolate": 1_000_000,
    "intersectFrustum": 1_000_000,
    "intersectSize": 1_000_000,
    "deform_setupPN+deform_getPN": 1_000_000,
    "rippleDeform": 1_000_000,
}
BIT_EXACT = set(COVERAGE) - {"deform_setupPN+deform_getPN", "rippleDeform"}


@pytest.fixture(scope="module")
def pin_results():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True, capture_output=True)
    if not os.path.exists(PIN):
        pytest.skip("reference checkout absent: oracle/_ref/ref_shader_pin not built")
    out = subprocess.run([PIN], capture_output=True, text=True, timeout=600)
    lines = [json.loads(line) for line in out.stdout.splitlines() if line.startswith("{")]
    return out.returncode, lines


def test_layouts_pinned_field_by_field(pin_results):
    """The pin program compiled, so every static_assert held: each field of the
    16 pinned shaderio structs has the offset and size of tc_<struct>'s."""
    _, lines = pin_results
    head = lines[0]
    assert head["layout_structs"] == 16
    assert head["layout_fields"] >= 200, head


def test_shader_functions_match_the_reference(pin_results):
    rc, lines = pin_results
    checks = {c["check"]: c for c in lines[1:]}
    assert set(checks) == set(COVERAGE), sorted(checks)
    for name, least in COVERAGE.items():
        c = checks[name]
        assert c["compared"] >= least, (name, c["compared"], least)
        assert c["mismatches"] == 0, c
        if name in BIT_EXACT:
            assert c["tolerance"] == 0 and c["max_err"] == 0, c
        else:
            assert c["max_err"] <= c["tolerance"] <= 2e-6, c
    assert rc == 0

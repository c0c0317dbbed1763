"""Arithmetic of the pixel shader compiled for the host from the kernels' own
headers (swegl_gb300/csrc/sgl_device.cuh, sgl_shade.cuh) and checked on
seeded inputs:

* sgl::spec_pow, the specular power, against the reference's
  (float)pow((double)s, p) (src/render/pixel_shaders.cpp:193).  The
  pair-of-floats exponentiation carries about 46 bits, so the rounded float
  differs from the reference's only where s^p lies within that error of a
  rounding boundary: a few in ten million draws, and then by one unit in the
  last place.
* sgl::light_sum, which skips lights clearly behind the surface before their
  division and normalisation, against the reference's loop taking every light
  through every step (src/render/pixel_shaders.cpp:159-205): equal bit for
  bit, including lights placed almost in the surface's tangent plane.
* sgl::cross_z_positive / cross_z_negative, the back-face and front-face
  tests, which decide the sign of the normalised cross product's z without
  its square root and division where that is provably the same, against the
  reference's normalised expression (src/projection/points.cpp:32-37), on
  ordinary, tiny, huge, subnormal, infinite and NaN edge vectors.
* The fused geometry pass's whole-primitive frustum test (sgl_cull.h):
  wherever it skips a primitive's box for a view, every vertex in the box,
  transformed as the pass transforms it, is in front of the camera and
  beyond the side the test found (inside_camera_frustum,
  src/render/renderer.cpp:58-70, rejects every triangle there); boxes are
  placed across and within 1e-6 of each side.  The same check with the
  test's rounding margin set to zero finds thousands of violations, so the
  placement reaches the margin."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "shade_math")


def _build(tmp, name):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out = str(tmp / name)
    subprocess.run([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "swegl_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
                    os.path.join(SRC, name + ".cu"), "-o", out], check=True)
    return out


@pytest.fixture(scope="module")
def exes(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("shade_math")
    return {n: _build(tmp, n) for n in ("spec_pow_host", "light_sum_host", "cross_sign_host", "cull_host")}


@pytest.mark.parametrize("pmax, allowed", [(128, 2e-6), (1024, 1e-5)])
def test_spec_pow_matches_double_pow(exes, pmax, allowed):
    r = subprocess.run([exes["spec_pow_host"], "3000000", str(pmax)], capture_output=True, text=True, check=True)
    used, diff, far = map(int, r.stdout.split())
    assert used > 1_000_000
    assert far == 0, f"{far} results off by more than one unit in the last place"
    assert diff <= allowed * used, f"{diff} of {used} differ from (float)pow((double)s, p)"


def test_light_sum_skips_only_lights_the_reference_skips(exes):
    r = subprocess.run([exes["light_sum_host"], "1000000"], capture_output=True, text=True, check=True)
    cases, diff, early, tangent = map(int, r.stdout.split())
    assert diff == 0, f"{diff} of {cases} light sums differ from the reference's loop"
    assert early > cases  # about half of the four lights per case are skipped early
    assert tangent == cases // 2


def test_cross_sign_matches_normalised_cross(exes):
    r = subprocess.run([exes["cross_sign_host"], "2000000"], capture_output=True, text=True, check=True)
    cases, diff = map(int, r.stdout.split())
    assert cases == 2000000 and diff == 0, f"{diff} of {cases} sign tests differ from the normalised cross product"


def test_primitive_frustum_test_skips_only_unseen_boxes(exes):
    r = subprocess.run([exes["cull_host"], "300000"], capture_output=True, text=True, check=True)
    boxes, skipped, vertices, bad = map(int, r.stdout.split())
    assert boxes == 300000
    assert skipped > boxes // 10 and vertices == 40 * skipped
    assert bad == 0, f"{bad} of {vertices} vertices of skipped boxes are not beyond the side the test found"

"""The `sequoia` command line tool and the C++ drop-in behind it
(sequoia_gb300/host): OBJ in, render.bmp out, against the reference's own
images (tests/golden) and the oracle."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

EXE = os.path.join(ROOT, "sequoia_gb300", "sequoia")


def _obj(tmp_path, tris):
    from sequoia_gb300 import scenes
    v = np.asarray(tris, np.float32).reshape(-1, 3)
    p = tmp_path / "scene.obj"
    scenes.write_obj(str(p), v, np.arange(len(v)).reshape(-1, 3))
    return str(p)


def _run(tmp_path, *args):
    r = subprocess.run([EXE, *args], capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ico3", "ico4", "soup3k"])
def test_cli_recursive_render_matches_reference(lib_built, tmp_path, name):
    """-builder recursive: the same tree as the reference's SAH builder, so
    render.bmp is byte-identical to the reference's image of that scene."""
    import sequoia_gb300 as sq
    g = load_golden(name)
    w, h = int(g["w"]), int(g["h"])
    out = _run(tmp_path, _obj(tmp_path, g["tris"]), "-builder", "recursive", "-res", str(w), str(h))
    assert "faces:        %d" % len(g["tris"]) in out
    assert (tmp_path / "render.bmp").read_bytes() == sq.encode_bmp(g["heat"], w, h)


@pytest.mark.gpu
@pytest.mark.parametrize("builder", ["morton", "grid", "grid_sse"])
def test_cli_other_builders_match_oracle(lib_built, oracle, tmp_path, builder):
    import sequoia_gb300 as sq
    g = load_golden("soup3k")
    tris = g["tris"]
    w, h = 96, 64
    _run(tmp_path, _obj(tmp_path, tris), "-builder", builder, "-res", str(w), str(h), "-o", "x.bmp")
    if builder == "morton":
        nodes, root = oracle.build_morton(tris)[:2]
    else:
        nodes, root = oracle.build_grid(tris, 8, 8, scene_bounds_cells=(builder == "grid"))[:2]
    rays = oracle.rays_reference_camera(w, h, g["cam"])
    _, _, tests = oracle.trace(nodes, root, tris, rays, 0)
    assert (tmp_path / "x.bmp").read_bytes() == sq.encode_bmp(oracle.heatmap(tests), w, h)


@pytest.mark.gpu
def test_cli_closest_mode_matches_oracle(lib_built, oracle, tmp_path):
    import sequoia_gb300 as sq
    g = load_golden("ico4")
    tris = g["tris"]
    w, h = 120, 90
    _run(tmp_path, _obj(tmp_path, tris), "-builder", "recursive", "-leaf", "4", "-bins", "16", "-mode", "closest",
         "-res", str(w), str(h))
    nodes, root, _ = oracle.build_sah(tris, 16, 4)
    rays = oracle.rays_reference_camera(w, h, g["cam"])
    _, _, tests = oracle.trace(nodes, root, tris, rays, 1)
    assert (tmp_path / "render.bmp").read_bytes() == sq.encode_bmp(oracle.heatmap(tests), w, h)


@pytest.mark.gpu
def test_cli_benchmark_mode(lib_built, tmp_path):
    g = load_golden("ico3")
    out = _run(tmp_path, _obj(tmp_path, g["tris"]), "-benchmark")
    assert "build time" in out and "mrps" in out
    for k in (1, 2, 3):
        assert (tmp_path / ("benchmark%d.bmp" % k)).stat().st_size == 54 + 1920 * 3 * 1080


@pytest.mark.gpu
@pytest.mark.parametrize("tracer,k", [("packet", 8), ("packet", 4), ("bundle", 64), ("bundle", 16)])
def test_cli_packet_bundle_render_matches_reference(lib_built, tmp_path, tracer, k):
    """-tracer packet <k> / bundle <k>: the reference's images of the same
    scene, byte for byte."""
    import sequoia_gb300 as sq
    g = load_golden("ico4")
    w, h = int(g["w"]), int(g["h"])
    _run(tmp_path, _obj(tmp_path, g["tris"]), "-builder", "recursive", "-tracer", tracer, str(k), "-res", str(w),
         str(h))
    assert (tmp_path / "render.bmp").read_bytes() == sq.encode_bmp(g["%s%d_heat" % (tracer, k)], w, h)

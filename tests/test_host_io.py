"""Host side of the drop-in (include/sequoia_host.h): the OBJ loader and the
BMP writer against the reference's own loadOBJFromFile and image output.
No GPU needed."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

CASES = np.load(os.path.join(GOLDEN, "obj_cases.npz"))
NAMES = sorted(k[:-5] for k in CASES.files if k.endswith("_text"))


@pytest.fixture(scope="module")
def sq(lib_built):
    import sequoia_gb300
    return sequoia_gb300


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("threads", [1, 4])
def test_obj_parse_matches_reference_golden(sq, name, threads):
    """Bit-identical triangles for every golden text (the reference's parse:
    fgets lines of 255 characters, gstrtok tokens, atof -> float, quads,
    negative and forward indices, CRLF, empty tokens)."""
    text = CASES[name + "_text"].tobytes()
    want = CASES[name + "_tris"]
    tris, info = sq.parse_obj(text, threads=threads)
    assert tris.shape == want.shape
    assert tris.tobytes() == want.tobytes()  # bytes: NaN coordinates compare equal
    assert info["faces"] == len(want)


def test_obj_load_file(sq, tmp_path):
    text = CASES["random_soup_text"].tobytes()
    p = tmp_path / "soup.obj"
    p.write_bytes(text)
    tris, info = sq.load_obj(str(p))
    assert tris.tobytes() == CASES["random_soup_tris"].tobytes()
    assert info["vertices"] == 3000


def _big_obj(nv=120000, seed=3):
    """About 6 MB of OBJ (several parse chunks) with negative and positive
    indices, quads and comments."""
    rng = np.random.default_rng(seed)
    v = (rng.standard_normal((nv, 3)) * 100).astype(np.float32)
    parts, emitted = [], 0
    for i in range(0, nv, 1000):
        blk = v[i:i + 1000]
        parts.append("".join("v %.9g %.9g %.9g\n" % tuple(map(float, r)) for r in blk))
        emitted += len(blk)
        k = rng.integers(1, emitted + 1, (600, 4))
        neg = rng.random((600, 4)) < 0.5
        quad = rng.random(600) < 0.25
        lines = []
        for row, ng, q in zip(k, neg, quad):
            toks = [str(int(a) - emitted - 1) if n else str(int(a)) for a, n in zip(row, ng)]
            lines.append("f " + " ".join(toks[:4 if q else 3]) + "\n")
        parts.append("# block %d\n" % i)
        parts.append("".join(lines))
    return "".join(parts).encode()


def test_obj_parallel_parse_independent_of_threads(sq):
    text = _big_obj()
    a, ia = sq.parse_obj(text, threads=1)
    b, ib = sq.parse_obj(text, threads=16)
    assert a.tobytes() == b.tobytes()
    assert ia["lines"] == ib["lines"] and ia["vertices"] == 120000


def test_obj_big_matches_reference(sq, oracle, tmp_path):
    if not oracle.ref_available("b8"):
        pytest.skip("reference library not built here")
    text = _big_obj()
    p = tmp_path / "big.obj"
    p.write_bytes(text)
    want = oracle.ref_load_obj(str(p))
    got, _ = sq.load_obj(str(p), threads=8)
    assert got.tobytes() == want.tobytes()


@pytest.mark.parametrize("text,where", [
    (b"v 1 2 3\nv 1 2\n", "line 2"),                       # missing token (the reference reads NULL)
    (b"v 1 2 3\nv 4 5 6\nv 7 8 9\nf 1 2 3", "line 4"),     # last index not delimited
    (b"v 1 2 3\nv 4 5 6\nv 7 8 9\nf 1 2 4\n", "line 4"),   # index past the vertex list
    (b"v 1 2 3\nv 4 5 6\nv 7 8 9\nf 0 1 2\n", "line 4"),   # index 0
    (b"v 1 2 3\nf -2 -1 1\n", "line 2"),                    # relative index before the first vertex
])
def test_obj_rejects_undefined_inputs(sq, text, where):
    with pytest.raises(sq.SequoiaError) as e:
        sq.parse_obj(text)
    assert where in str(e.value)


def test_obj_missing_file(sq, tmp_path):
    with pytest.raises(sq.SequoiaError):
        sq.load_obj(str(tmp_path / "nope.obj"))


@pytest.mark.parametrize("w,h", [(1, 1), (7, 5), (8, 3), (161, 121)])
def test_bmp_matches_reference(sq, oracle, tmp_path, w, h):
    rgb = np.random.default_rng(w * 1000 + h).integers(0, 256, w * h * 3, dtype=np.uint8)
    data = sq.encode_bmp(rgb, w, h)
    p = tmp_path / "a.bmp"
    sq.write_bmp(str(p), rgb, w, h)
    assert p.read_bytes() == data
    if oracle.ref_available("b8"):
        q = tmp_path / "ref.bmp"
        oracle.ref_write_bmp(str(q), w, h, rgb)
        assert q.read_bytes() == data
    # the format itself: 54-byte header, B G R rows padded to 4 bytes, rgb row 0 first
    row = (3 * w + 3) & ~3
    assert len(data) == 54 + row * h
    assert int.from_bytes(data[2:6], "little") == len(data)
    px = np.frombuffer(data[54:], np.uint8).reshape(h, row)[:, :3 * w].reshape(h, w, 3)
    assert np.array_equal(px[..., ::-1], rgb.reshape(h, w, 3))


def test_golden_heatmap_bmp(sq, oracle):
    """The reference's render.bmp of a golden heatmap, byte for byte."""
    if not oracle.ref_available("b8"):
        pytest.skip("reference library not built here")
    import tempfile
    g = np.load(os.path.join(GOLDEN, "ico3.npz"))
    w, h = int(g["w"]), int(g["h"])
    with tempfile.TemporaryDirectory() as d:
        q = os.path.join(d, "r.bmp")
        oracle.ref_write_bmp(q, w, h, g["heat"])
        assert open(q, "rb").read() == sq.encode_bmp(g["heat"], w, h)


def test_cli_usage(lib_built):
    import subprocess
    exe = os.path.join(ROOT, "sequoia_gb300", "sequoia")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "Usage" in r.stdout


def test_cli_missing_file_exits_1(lib_built, tmp_path):
    """As the reference: "Can't open OBJ file" on stderr, exit status 1
    (before any GPU work)."""
    import subprocess
    exe = os.path.join(ROOT, "sequoia_gb300", "sequoia")
    r = subprocess.run([exe, str(tmp_path / "none.obj")], capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and "Can't open OBJ file" in r.stderr

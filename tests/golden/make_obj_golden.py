"""Golden OBJ parses: edge-case OBJ texts and the triangles the reference's
own loadOBJFromFile (src/main.cpp:108-179) returns for them.

Run where oracle/_ref was built (x86-64 with the reference tree):
    python tests/golden/make_obj_golden.py
Writes tests/golden/obj_cases.npz: for each case `<name>_text` (uint8 bytes
of the file) and `<name>_tris` (float32 (n, 9)).  Every text is one the
reference parses without undefined behaviour (no missing tokens, no index
outside the vertex list): those inputs have no reference answer.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle.oracle as O  # noqa: E402


def cases():
    rng = np.random.default_rng(11)
    c = {}
    c["plain"] = b"v 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nf 1 2 3\nf 1 3 4\n"
    c["quads_negative"] = (b"v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3 4\n"
                           b"v 0 0 2\nv 1 0 2\nv 1 1 2\nf -1 -2 -3\nf -4 -3 -2 -1\nf 1 2 3 4 5\n")
    c["slashes_comments"] = (b"# header\n#no space comment\no thing\ng group\ns 1\nusemtl m\n"
                             b"v 1.5 -2.25 3e2\nvt 0.5 0.5\nvn 0 0 1\nv -1e-3 0x1p-3 7.0000001\n"
                             b"v 2.5abc 4 5\nf 1/1/1 2/1/1 3/1/1\nf 3//1 2//1 1//1\n\n\n")
    c["tabs_crlf"] = b"v\t1\t2\t3\r\nv 4 5 6\r\nv 7\t8 9\r\n\r\nf 1 2 3\r\nf\t3 2 1\r\n"
    c["empty_tokens"] = b"v  1 2 3\nv 4  5 6\nv 7 8 9\nf 1 2 3\n"  # double spaces read as 0
    c["forward_refs"] = b"f 1 2 3\nf 2 3 4\nv 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 1\n"
    c["no_final_newline_quad"] = b"v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nf 1 2 3 4"
    # a 255-character fgets() line ends mid-comment; the rest of the line is
    # read as a line of its own, which here is a vertex record
    c["long_line_split"] = (b"v 0 0 0\nv 1 0 0\n# " + b"x" * 253 + b"v 0 1 0\nf 1 2 3\n")
    c["long_trailing_spaces"] = b"v 0 0 0 " + b" " * 300 + b"\nv 1 0 0\nv 0 1 0\nf 1 2 3\n"
    c["nul_in_comment"] = b"v 0 0 0\n# a\x00b\nv 1 0 0\nv 0 1 0\nf 1 2 3\n"
    c["special_values"] = b"v inf -inf 1\nv 1e39 -1e-46 nan\nv 3.4028235e38 1.17549435e-38 1.4e-45\nf 1 2 3\n"
    c["no_faces"] = b"v 1 2 3\n# nothing else\n"
    c["empty"] = b""
    # random soup: %.9g round-trips float32; negative and positive indices
    nv = 3000
    v = rng.standard_normal((nv, 3)).astype(np.float32) * np.float32(10)
    lines = []
    emitted = 0
    for i in range(nv):
        lines.append(b"v %.9g %.9g %.9g\n" % tuple(float(x) for x in v[i]))
        emitted += 1
        if emitted >= 4 and rng.random() < 0.7:
            idx = rng.integers(1, emitted + 1, 4)
            toks = [(b"%d" % k) if rng.random() < 0.5 else (b"%d" % (k - emitted - 1)) for k in idx]
            n = 4 if rng.random() < 0.3 else 3
            lines.append(b"f " + b" ".join(toks[:n]) + b"\n")
    c["random_soup"] = b"".join(lines)
    return c


def main():
    if not O.ref_available("b8"):
        sys.exit("oracle/_ref/libseqref_b8.so is not built (oracle/build_ref.sh)")
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for name, text in cases().items():
            path = os.path.join(d, name + ".obj")
            with open(path, "wb") as fh:
                fh.write(text)
            tris = O.ref_load_obj(path)
            out[name + "_text"] = np.frombuffer(text, np.uint8).copy()
            out[name + "_tris"] = np.asarray(tris, np.float32).reshape(-1, 9)
            print(name, len(text), "bytes ->", len(out[name + "_tris"]), "triangles")
    np.savez_compressed(os.path.join(HERE, "obj_cases.npz"), **out)


if __name__ == "__main__":
    main()

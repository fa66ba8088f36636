"""Wavefront OBJ texts for the loader's parity tests: hand-written edge cases of the reference's
line patterns (wavefront_obj::load_geometry, resource.cpp:137-255) and a seeded random generator.
"""
import numpy as np

QUAD = ("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\nvn 0 0 1\n"
        "f 1/1/1 2/2/1 3/3/1\nf 3/3/1 4/4/1 1/1/1\n")

CASES = {
    "quad": QUAD,
    "crlf": QUAD.replace("\n", "\r\n"),
    "no_final_newline": QUAD.rstrip("\n"),
    "spaces_tabs": ("v  0.5\t-1.25   2\t \nv 1 2 3  \nv\t4 5 6\r\nvt 0.25  0.75 \nvn 0 1 0\n"
                    "f  1/1/1\t2/1/1  3/1/1 \n"),
    "four_numbers": "v 1 2 3 4\nv 5 6 7\nv 8 9 10\nvt 0.5 0.25 0.125\nvn 1 0 0\nf 1/1/1 2/1/1 3/1/1\n",
    "other_lines": ("# comment\nmtllib x.mtl\no thing\ng grp\ns 1\nusemtl m\n\n v 9 9 9\nv 0 0 0\n"
                    "v 0 0 1\nv 0 1 0\nvx 1 2 3\nvt 0 0\nvn 1 0 0\nf 1/1/1 2/1/1 3/1/1\n"),
    "number_forms": ("v 1e3 -2.5E-2 0x1p-3\nv +7 007 .5\nv 3.4028234e38 -0.0 1.17549435e-38\nvt inf 0\n"
                     "vn nan -inf 2\nf 1/1/1 2/1/1 3/1/1\n"),
    "trailing_text": "v 1abc 2x 3 y\nv 0 0 0\nv 1 1 1\nvt 0 0\nvn 0 0 1\nf 1/1/1 2/1/1 3/1/1zz\n",
    "last_write_wins": ("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nvt 0.1 0.1\nvt 0.2 0.2\nvt 0.3 0.3\n"
                        "vn 1 0 0\nvn 0 1 0\nvn 0 0 1\nf 1/1/1 2/2/2 3/3/3\nf 2/3/3 4/1/2 3/2/1\n"),
    "unreferenced_vertex": "v 0 0 0\nv 1 0 0\nv 0 1 0\nv 5 5 5\nvt 0 0\nvn 0 0 1\nf 1/1/1 2/1/1 3/1/1\n",
    "vertices_only": "v 0 0 0\nv 1 0 0\n",
    "trailing_slash": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\nf 1/1/1/ 2/1/1/ 3/1/1/\n",
    "signs_in_index": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\nf +1/1/1 2/+1/1 3/1/+1\n",
    # errors
    "err_quad_face": QUAD + "f 1/1/1 2/1/1 3/1/1 4/1/1\n",
    "err_no_slashes": "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n",
    "err_zero_index": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\nf 0/1/1 2/1/1 3/1/1\n",
    "err_index_range": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\nf 1/1/1 2/1/1 4/1/1\n",
    "err_normal_range": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\nf 1/1/1 2/1/2 3/1/1\n",
    "err_forward_reference": "v 0 0 0\nv 1 0 0\nvt 0 0\nvn 0 0 1\nf 1/1/1 2/1/1 3/1/1\nv 0 1 0\n",
    "err_no_vertices": "vt 0 0\nvn 0 0 1\n# nothing\n",
    "err_empty": "",
    "err_overflow": "v 1e50 0 0\n",
    "err_underflow": "v 1e-40 0 0\n",
    "err_not_a_number": "v a b c\n",
    "err_three_spaces": "v   1 2\n",
    "err_four_parts": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\nf 1/1/1/1 2/1/1 3/1/1\n",
    "err_negative_index": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\nf -1/1/1 2/1/1 3/1/1\n",
    "err_no_normals": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nf 1/1/ 2/1/ 3/1/\n",
    "err_vertex_missing": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\nf /1/1 2/1/1 3/1/1\n",
}

# Faces whose corners omit a texcoord index ("a//c"): the reference reads out of bounds on them,
# so they are never given to it; the loader refuses them. (A corner without a normal index,
# "a/b/", splits into two pieces and is an error in the reference too.)
UNDEFINED_IN_REFERENCE = {
    "no_texcoords": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\n",
    "mixed": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\nf 1/1/1 2/1/1 3/1/1\nf 1//1 2//1 3//1\n",
}


def _num(rng, bad):
    k = rng.integers(8)
    x = rng.normal(0, 10)
    if k == 0:
        return f"{x:.3e}"
    if k == 1:
        return f"{x:+.2f}"
    if k == 2:
        return str(int(x))
    if k == 3:
        return f"{x:.9g}"
    if k == 4:
        return str(rng.choice(["0", "-0", ".5", "5.", "1e-3", "0x1.8p1", "inf", "nan", "2.5f", "7e+1"]
                              + (["1e40", "q", "-", "1e-45"] if bad else [])))
    return f"{x:.6f}"


def _sep(rng):
    return str(rng.choice([" ", " ", " ", "  ", "\t", " \t"] + ["   "] * (rng.random() < 0.02)))


def random_obj(rng, lines=24):
    """A random OBJ text: every kind of line with varied whitespace, number spellings and line
    ends; about one file in four also holds a malformed line or index."""
    bad = rng.random() < 0.25
    out = []
    nv = nt = nn = 0
    for _ in range(lines):
        k = int(rng.integers(10))
        if nv < 3 or nt < 1 or nn < 1:
            k = [0, 4, 3][int(np.argmin([nv - 2, nt, nn]))]
        end = str(rng.choice(["", "", "", " ", "\r", " \r", "\t"]))
        if k <= 2:
            cnt = 3 if (not bad or rng.random() < 0.9) else int(rng.integers(1, 6))
            if cnt == 3 and rng.random() < 0.05:
                cnt = 4  # the first group takes two numbers
            out.append("v" + "".join(_sep(rng) + _num(rng, bad) for _ in range(cnt)) + end)
            nv += 1
        elif k == 3:
            out.append("vn" + "".join(_sep(rng) + _num(rng, bad) for _ in range(3)) + end)
            nn += 1
        elif k == 4:
            cnt = 2 if rng.random() < 0.8 else 3
            out.append("vt" + "".join(_sep(rng) + _num(rng, bad) for _ in range(cnt)) + end)
            nt += 1
        elif k <= 7:
            corners = 3 if (not bad or rng.random() < 0.9) else 4

            def idx(n):
                hi = n + (2 if bad else 1)
                return str(int(rng.integers(1, max(hi, 2))))
            cs = [f"{idx(nv)}/{idx(nt)}/{idx(nn)}" for _ in range(corners)]
            out.append("f" + "".join(_sep(rng) + c for c in cs) + end)
        else:
            out.append(str(rng.choice(["# c", "", "o x", "s off", "vx 1 2 3", " v 1 2 3", "usemtl a", "g"])))
    return "\n".join(out) + ("\n" if rng.random() < 0.7 else "")


def pack_texts(texts):
    """Concatenated bytes and offsets (fixtures hold no pickled objects)."""
    raw = [t.encode() for t in texts]
    off = np.concatenate([[0], np.cumsum([len(r) for r in raw])]).astype(np.int64)
    return np.frombuffer(b"".join(raw), np.uint8).copy(), off


def unpack_texts(data, off):
    return [bytes(data[off[i]:off[i + 1]]).decode() for i in range(len(off) - 1)]

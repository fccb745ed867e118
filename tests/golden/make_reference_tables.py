"""Writes reference_tables.json: the integer tables that accelerate-fourier's
own source documents in comments, read from the reference source tree.

  - src/Data/Array/Accelerate/Fourier/Planned.hs: the Fourier exponent matrix
    of size 7, its multiplicative generator, the permutation by powers of the
    generator, the permuted matrix and the inverse permutation (Rader);
  - src/Data/Array/Accelerate/Fourier/Private.hs: the exponent matrix of size
    5, the permutation `Permutation.T` and the permuted matrix (transform5).

The fixture is committed; the tests read it and never the reference tree.
Run from the repository root:  python tests/golden/make_reference_tables.py REFERENCE_ROOT
(REFERENCE_ROOT: the root of the accelerate-fourier source tree)
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def comment_blocks(path):
    """(first line number, lines) of every {- ... -} block comment."""
    lines = open(path).read().split("\n")
    out, cur, start = [], None, 0
    for i, line in enumerate(lines, 1):
        t = line.strip()
        if cur is None and t.startswith("{-") and not t.startswith("{-#") and "-}" not in t:
            cur, start = [], i
            continue
        if cur is not None:
            if line.strip().startswith("-}"):
                out.append((start, cur))
                cur = None
            else:
                cur.append((i, line))
    return out


def matrices(block):
    """Runs of lines that hold only integers, with their first line number."""
    mats, cur = [], []
    for num, line in block:
        if re.fullmatch(r"\s*\d+(\s+\d+)+\s*", line):
            cur.append((num, [int(t) for t in line.split()]))
        elif cur:
            mats.append(cur)
            cur = []
    if cur:
        mats.append(cur)
    return [(m[0][0], m[-1][0], [r for _, r in m]) for m in mats]


def labelled(block, label):
    for num, line in block:
        if label in line:
            return num, [int(t) for t in re.findall(r"\d+", line.split(":", 1)[1])]
    raise KeyError(label)


def main(root):
    planned = "src/Data/Array/Accelerate/Fourier/Planned.hs"
    private = "src/Data/Array/Accelerate/Fourier/Private.hs"
    out = {}
    for start, block in comment_blocks(os.path.join(root, planned)):
        if any("Fourier exponent matrix of a signal of size 7" in l for _, l in block):
            mats = matrices(block)
            gl, gen = labelled(block, "multiplicative generator in Z7")
            pl, perm = labelled(block, "permutation of rows and columns by powers of 3")
            il, inv = labelled(block, "Inverse permutation")
            out["rader7"] = {
                "source": f"{planned}:{start}-{il}",
                "exponent_matrix": mats[0][2], "generator": gen[-1], "powers": perm,
                "permuted_matrix": mats[1][2], "inverse": inv,
            }
    for start, block in comment_blocks(os.path.join(root, private)):
        if any("Permutation.T" in l for _, l in block):
            mats = matrices(block)
            tl, perm = labelled(block, "Permutation.T")
            out["small5"] = {
                "source": f"{private}:{start}-{mats[-1][1]}",
                "exponent_matrix": mats[0][2], "permutation": perm, "permuted_matrix": mats[1][2],
            }
    assert set(out) == {"rader7", "small5"}, sorted(out)
    with open(os.path.join(HERE, "reference_tables.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_reference_tables.py REFERENCE_ROOT  (the accelerate-fourier source tree)")
    main(sys.argv[1])

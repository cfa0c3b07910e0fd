"""Writes tests/golden/warp3d_test24.npz from WARP3D's own regression
problem verification/test24 (the hollow sphere under internal pressure:
45 finite-strain b-bar 8-node bricks, bilinear Mises, skew constraints,
nodal forces in 21 steps) and the answer its checker expects
(verification/test24/driver.inp: the first stress value printed for
element 1 after step 21, checked to 1e-4 by verification/run_tests.py).

Run in a checkout that has the WARP3D sources next to this repository:
    python -m tests.golden.make_warp3d_test24 <path to WARP3D>/verification/test24

The fixture holds the deck's data as arrays; the test that uses it runs
on any machine without the WARP3D tree.
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "warp3d_test24.npz")


def _lines(path):
    """Deck lines without comments ('c' in column 1 followed by a blank, or
    a lone 'c') and without '$' trailers, continuation commas kept."""
    out = []
    for raw in open(path):
        s = raw.rstrip("\n")
        if re.match(r"^\s*c(\s|$)", s, flags=re.IGNORECASE) or not s.strip():
            continue
        s = s.split("$")[0].rstrip()
        if s.strip():
            out.append(s.strip())
    return out


def _join_continued(lines, i):
    """Joins a statement whose lines end with ',' (WARP3D continuation)."""
    text = lines[i]
    while text.endswith(","):
        i += 1
        text = text[:-1] + " " + lines[i]
    return text, i


def _ints(words):
    return [int(w) for w in words if re.fullmatch(r"\d+", w)]


def parse(deck):
    L = _lines(deck)
    d = {}
    i = 0
    trn_nodes, trn_mats, trn_fixed = [], [], []
    planes = []
    loads = {}
    steps = []
    while i < len(L):
        s = L[i]
        low = s.lower()
        if low.startswith("properties bilinear"):
            w = low.split()
            d["props"] = np.array([float(w[w.index(k) + 1]) for k in ("e", "nu", "yld_pt", "tan_e")])
        elif low.startswith("number of nodes"):
            nnode = int(low.split()[-1])
        elif low.startswith("number of elements"):
            nelem = int(low.split()[-1])
        elif low == "coordinates":
            xyz = np.zeros((nnode, 3))
            for k in range(nnode):
                w = L[i + 1 + k].split()
                xyz[int(w[0]) - 1] = [float(v) for v in w[1:4]]
            d["coords"] = xyz
            i += nnode
        elif low == "elements":   # the options follow on the next (continued) lines
            stmt, i = _join_continued(L, i + 1)
            t = stmt.lower()
            d["flags"] = np.array([int("nonlinear" in t), int("bbar" in t), int("center_output" in t)])
        elif low == "incidences":
            inc = np.zeros((nelem, 8), dtype=np.int64)
            for k in range(nelem):
                w = L[i + 1 + k].split()
                inc[int(w[0]) - 1] = [int(v) for v in w[1:9]]
            d["incid"] = inc - 1
            i += nelem
        elif low.startswith("transformation matrix"):
            # one continued statement: the node list, then row_1..row_3
            stmt, i = _join_continued(L, i)
            w = stmt.replace(",", " ").split()
            r1 = [x.lower() for x in w].index("row_1")
            nodes = _ints(w[2:r1])
            rows = []
            for r in range(3):
                k = [x.lower() for x in w].index(f"row_{r + 1}")
                rows.append([float(v) for v in w[k + 1:k + 4]])
            con, i = _join_continued(L, i + 1)
            w = con.split()
            fixed = [c for c in "uvw" if c in [x.lower() for x in w]]
            for c in fixed:
                k = [x.lower() for x in w].index(c)
                assert float(w[k + 1]) == 0.0
            cnodes = _ints(w[:[x.lower() for x in w].index(fixed[0])])
            assert sorted(cnodes) == sorted(nodes)
            trn_nodes.append(np.array(nodes) - 1)
            trn_mats.append(np.array(rows))
            trn_fixed.append(np.array(["uvw".index(c) for c in fixed]))
        elif low.startswith("plane") and "symmetry" in low:
            w = low.split()
            planes.append(("xyz".index(w[1]), float(w[3])))
        elif low.startswith("loading unit_press"):
            k = i + 2   # 'nodal loads'
            assert L[i + 1].lower() == "nodal loads"
            while k < len(L) and "force_x" in L[k]:
                w = L[k].split()
                loads[int(w[0]) - 1] = [float(w[2]), float(w[4]), float(w[6])]
                k += 1
            i = k - 1
        elif low.startswith("step "):
            w = low.split()
            rng = w[1].split("-")
            a, b = int(rng[0]), int(rng[-1])
            steps += [float(w[3])] * (b - a + 1)
        i += 1
    F = np.zeros((nnode, 3))
    for n, f in loads.items():
        F[n] = f
    d["load_pattern"] = F
    d["step_factors"] = np.array(steps)
    d["trn_mats"] = np.array(trn_mats)
    d["trn_node_lists"] = np.concatenate(trn_nodes)
    d["trn_counts"] = np.array([len(x) for x in trn_nodes])
    d["trn_fixed"] = np.array([[int(k in f) for k in range(3)] for f in trn_fixed])
    # symmetry planes: the nodes on the plane (to 1e-6 of the model size)
    # have the plane-normal displacement fixed
    scale = np.abs(d["coords"]).max()
    d["plane_fixed_dofs"] = np.array(sorted(
        3 * n + ax for ax, val in planes for n in np.nonzero(np.abs(d["coords"][:, ax] - val) <= 1e-6 * scale)[0]))
    return d


def expected(driver):
    """The answer the checker compares and the element / step it is read
    from (verification/run_tests.py format: search lines, skip, answer,
    word position)."""
    L = [s.strip() for s in open(driver) if s.strip() and not s.lstrip().startswith(("#", "*"))]
    ans = float(L[-2])
    pos = int(L[-1])
    return ans, pos


def main(test_dir):
    d = parse(os.path.join(test_dir, "test_24"))
    ans, pos = expected(os.path.join(test_dir, "driver.inp"))
    d["expected_answer"] = np.array(ans)
    d["expected_word"] = np.array(pos)
    np.savez_compressed(OUT, **d)
    print(OUT, {k: np.shape(v) for k, v in d.items()}, ans)


if __name__ == "__main__":
    main(sys.argv[1])

"""Writes tests/golden/warp3d_test82_voce.npz from WARP3D's own regression
problem verification/test82/voche_model (mm10 crystal plasticity: 208
small-displacement b-bar 8-node bricks on the unit cube, one bcc crystal
of fixed orientation, Voce hardening, symmetry planes, element face
pressures in 10 steps of 50) and the answer its checker expects
(verification/test82/voche_model/driver.inp: the first stress printed for
element 64 after step 8, checked to 1e-4 by verification/run_tests.py).

Run in a checkout that has the WARP3D sources next to this repository:
    python -m tests.golden.make_warp3d_test82_voce <path to WARP3D>/verification/test82/voche_model
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "warp3d_test82_voce.npz")


def _statements(path):
    """Deck statements: comments ('!' or 'c ' lines, '$' trailers) dropped,
    lines ending in ',' joined with the next."""
    out, cur = [], ""
    for raw in open(path):
        s = raw.rstrip("\n")
        if s.lstrip().startswith(("!", "*")) or re.match(r"^\s*c(\s|$)", s, flags=re.IGNORECASE):
            continue
        s = s.split("$")[0].strip()
        if not s:
            continue
        cur = (cur + " " + s).strip() if cur else s
        if cur.endswith(","):
            cur = cur[:-1]
            continue
        out.append(cur)
        cur = ""
    return out


def _value(words, key):
    low = [w.lower() for w in words]
    return words[low.index(key) + 1]


def parse(deck):
    S = _statements(deck)
    d = {}
    i = 0
    face_loads, planes = [], []
    while i < len(S):
        s = S[i]
        low = s.lower()
        w = s.replace(",", " ").split()
        if low.startswith("crystal "):
            props = " ".join(S[i + 1:i + 4]).replace(",", " ").split()   # slip_type ... tau_v
            assert _value(props, "slip_type").lower() == "bcc"
            assert _value(props, "elastic_type").lower() == "isotropic"
            assert _value(props, "hardening").lower() == "voce"
            d["crystal"] = np.array([float(_value(props, k).rstrip("."))
                                     for k in ("e", "nu", "harden_n", "voce_m", "theta_0", "tau_y", "tau_v")])
        elif low.startswith("properties cp"):
            mat = " ".join(S[i:i + 5]).replace(",", " ").split()
            assert _value(mat, "angle_convention").lower() == "kocks"
            assert _value(mat, "angle_type").lower() == "degrees"
            assert _value(mat, "n_crystals") == "1"
            k = [x.lower() for x in mat].index("angles")
            d["angles"] = np.array([float(x) for x in mat[k + 1:k + 4]])
        elif low.startswith("number of nodes"):
            nnode, nelem = int(w[3]), int(w[5])
        elif low == "coordinates":
            xyz = np.zeros((nnode, 3))
            k = i + 1
            n = 0
            while n < nnode:
                t = S[k].split()
                if len(t) == 4 and re.fullmatch(r"\d+", t[0]):
                    xyz[int(t[0]) - 1] = [float(v) for v in t[1:]]
                    n += 1
                k += 1
            d["coords"] = xyz
            i = k - 1
        elif low == "elements":
            t = S[i + 1].lower()
            d["flags"] = np.array([int("nonlinear" in t), int("bbar" in t), int("center_output" in t)])
        elif low == "incidences":
            inc = np.zeros((nelem, 8), dtype=np.int64)
            k = i + 1
            n = 0
            while n < nelem:
                t = S[k].split()
                if len(t) == 9 and re.fullmatch(r"\d+", t[0]):
                    inc[int(t[0]) - 1] = [int(v) for v in t[1:]]
                    n += 1
                k += 1
            d["incid"] = inc - 1
            i = k - 1
        elif low.startswith("plane") and "symmetry" in low:
            m = re.match(r"plane\s+([xyz])\s*=\s*([-+0-9.eE]+)\s+symmetry", low)
            planes.append(("xyz".index(m.group(1)), float(m.group(2))))
        elif re.match(r"^\d+\s+face\s+\d+\s+pressure", low):
            face_loads.append([int(w[0]) - 1, int(w[2]), float(w[4])])
        elif low.startswith("step ") and "unit_biaxial" in low:
            a, b = (int(x) for x in w[1].split("-"))
            d["step_factors"] = np.full(b - a + 1, float(w[3]))
        elif low.startswith("time step"):
            d["dt"] = np.array(float(w[2]))
        elif low.startswith("compute displacements") and "step" in low:
            d["last_step"] = np.array(int(w[-1]))
        i += 1
    d["face_loads"] = np.array(face_loads)
    scale = np.abs(d["coords"]).max()
    d["plane_fixed_dofs"] = np.array(sorted(
        3 * n + ax for ax, val in planes for n in np.nonzero(np.abs(d["coords"][:, ax] - val) <= 1e-6 * scale)[0]))
    return d


def expected(driver):
    """Element and value of the checker's answer (search line ' 64      1 ',
    skip 0, answer, word position)."""
    L = [s.strip() for s in open(driver) if s.strip() and not s.lstrip().startswith(("#", "*"))]
    search = L[-4].strip("'").split()
    return int(search[0]), float(L[-2]), int(L[-1])


def main(test_dir):
    d = parse(os.path.join(test_dir, "warp3d_voche.inp"))
    elem, ans, pos = expected(os.path.join(test_dir, "driver.inp"))
    d["expected_element"] = np.array(elem - 1)
    d["expected_answer"] = np.array(ans)
    d["expected_word"] = np.array(pos)
    np.savez_compressed(OUT, **d)
    print(OUT, {k: np.shape(v) for k, v in d.items()}, elem, ans, pos)


if __name__ == "__main__":
    main(sys.argv[1])

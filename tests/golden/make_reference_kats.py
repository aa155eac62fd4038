"""Extracts the known-answer vectors of the reference's own tests into reference_kats.json.

Reads (as text) the reference project's tests:
  tests/simulation/test_LinearAlgebra.cpp   angles_to_unit_vectors KAT (lines 13-40)
  tests/simulation/test_EuclideanTiling.cpp seam-wrap KAT (lines 41-73)
  tests/simulation/test_Locomotion.cpp      (commented out in the reference) repulsive_adhesion (42-60),
                                            mean angle (63-82), symmetrisation (87-136),
                                            get_dist_vect (141-263), average n (279-335)
Run from the repository root:  python tests/golden/make_reference_kats.py <path to the reference checkout>
"""
import json
import math
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_reference_kats.py <path to the reference checkout>")
REF = sys.argv[1]
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def uncomment(src):
    lines = []
    for ln in src.splitlines():
        s = ln.lstrip()
        while s.startswith("//"):
            s = s[2:].lstrip()
        lines.append(s)
    return "\n".join(lines)


def block(src, start_pat, end_pat):
    i = src.index(start_pat)
    j = src.index(end_pat, i + len(start_pat))
    return src[i:j]


NUM = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?"


def init_list(src, name):
    """Numbers of the Eigen comma initializer `name << a, b, ...;`."""
    m = re.search(r"\b" + re.escape(name) + r"\s*<<(.*?);", src, re.S)
    if not m:
        raise KeyError(name)
    return [float(x) for x in re.findall(NUM, m.group(1))]


def main():
    out = {"source": "reference tests/simulation/*.cpp (extracted as text)"}

    la = read("tests/simulation/test_LinearAlgebra.cpp")
    deg = [int(x) for x in init_list(la, "avg_n")]
    exp = {}
    for m in re.finditer(r"ASSERT_NEAR\(n_vec\((\d+),\s*(\d+)\),\s*([^,]+),\s*(" + NUM + r")\)", la):
        i, j, expr = int(m.group(1)), int(m.group(2)), m.group(3)
        exp[(i, j)] = float(eval(expr, {"sqrt": math.sqrt}))
        tol = float(m.group(4))
    out["angles_to_unit_vectors"] = dict(deg=deg, expected=[[exp[(i, 0)], exp[(i, 1)]] for i in range(len(deg))],
                                         tol=tol)

    et = read("tests/simulation/test_EuclideanTiling.cpp")
    out["seam_wrap"] = dict(uv_old=init_list(et, "r_UV_old"), uv=init_list(et, "r_UV"),
                            n=[int(x) for x in init_list(et, "n")], expected=init_list(et, "expected"),
                            tol=float(re.search(r"EPSILON\s*=\s*(" + NUM + ")", et).group(1)))

    lo = uncomment(read("tests/simulation/test_Locomotion.cpp"))
    fx = block(lo, "class LocomotionTest", "};")
    k = float(re.search(r"k\((" + NUM + r")\)", fx).group(1))
    sigma = float(re.search(r"σ\((" + NUM + r")\)", fx).group(1))
    r_adh = float(re.search(r"r_adh\((" + NUM + r")\)", fx).group(1))
    k_adh = float(re.search(r"k_adh\((" + NUM + r")\)", fx).group(1))
    rep = []
    for name in ("RepulsiveAdhesionTest1", "RepulsiveAdhesionTest2"):
        b = block(lo, name, "TEST_F")
        dv = [float(x) for x in re.findall(NUM, re.search(r"dist_v\((.*?)\);", b).group(1))]
        dist = float(re.search(r"double dist = (" + NUM + ")", b).group(1))
        ex = [float(x) for x in re.findall(NUM, re.search(r"expected_result\((.*?)\);", b).group(1))]
        rep.append(dict(dist_v=dv, dist=dist, expected=ex))
    out["repulsive_adhesion"] = dict(k=k, sigma=sigma, r_adh=r_adh, k_adh=k_adh, cases=rep, tol=1e-5)

    ma = []
    for name in ("CorrectlyCalculatesMeanAngle", "CorrectlyHandlesNegativeAngles"):
        b = block(lo, name, "TEST_F")
        angles = [float(x) for x in re.findall(NUM, re.search(r"angles\s*\{(.*?)\}", b).group(1))]
        e = float(re.search(r"expected_mean_angle = (" + NUM + ")", b).group(1))
        ma.append(dict(angles=angles, expected=e))
    out["mean_angle"] = dict(cases=ma, tol=1e-5, empty_throws=True)

    sym = []
    for name in ("SymmetricMatrixTestBasicTest", "SymmetricMatrixTestZeroTest", "SymmetricMatrixTestAllZerosTest"):
        b = block(lo, name, "TEST_F")
        sym.append(dict(mat=init_list(b, "mat"), expected=init_list(b, "expected_mat")))
    out["symmetrize_min"] = dict(cases=sym)

    dvc = []
    for name in ("GetDistVectTestBasicTest", "GetDistVectTestZeroMatrixTest", "GetDistVectTestOneDimensionTest",
                 "GetDistVectTestHandlesSquareMatrixCorrectly", "GetDistVectTestTenDimensionTest"):
        b = block(lo, name, "TEST_F" if name != "GetDistVectTestTenDimensionTest" else "CompareMatrices")
        r = init_list(b, "r")
        if "expected_diff_x" in b:
            ex, ey = init_list(b, "expected_diff_x"), init_list(b, "expected_diff_y")
        else:
            ex = ey = init_list(b, "expected_diff")
        dvc.append(dict(r=r, dx=ex, dy=ey))
    out["dist_vect"] = dict(cases=dvc, tol=1e-5)

    b = block(lo, "AverageNWithinDistanceTest1", "int main")
    out["average_n"] = dict(sigma=float(re.search(r"double σ = (" + NUM + ")", b).group(1)),
                            dist_length=init_list(b, "dist_length"), n=[int(x) for x in init_list(b, "n")],
                            expected=[int(x) for x in init_list(b, "expected_n")], tol=2)

    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()

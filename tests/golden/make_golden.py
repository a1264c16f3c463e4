"""Extracts the reference's own known-answer test data into reference_cases.json.

rulinalg is Rust and cannot be built or imported here, so its golden vectors are its
test sources: this script reads the `matrix![..]`, `vector![..]` and `vec![..]` literals
(and a few scalar expectations) at the cited file:line ranges of the reference checkout
and writes them, with their citations, as a JSON fixture. Run it where the reference is
present:

    python tests/golden/make_golden.py /path/to/rulinalg

The fixture is committed; tests never read the reference tree.
"""
from __future__ import annotations

import json
import re
import sys
from fractions import Fraction
from pathlib import Path

HERE = Path(__file__).resolve().parent


def _num(tok: str) -> float:
    tok = tok.strip().replace("- ", "-")
    tok = re.sub(r"(f32|f64|usize|i32|u32|u64)$", "", tok)
    tok = re.sub(r"(\d)(f32|f64|usize)", r"\1", tok)
    if not re.fullmatch(r"[-+0-9.eE/ ]+", tok):
        raise ValueError(f"unexpected literal element {tok!r}")
    if "/" in tok:
        a, b = tok.split("/")
        return float(Fraction(a.replace(" ", "")) / Fraction(b.replace(" ", "")))
    return float(tok)


def _literals(text: str):
    """All matrix!/vector!/vec! literals in order. Doc-test lines (`///`, `/// #`) count,
    plain `//` comment lines are skipped."""
    kept = []
    for line in text.splitlines():
        t = line.lstrip()
        if t.startswith("///"):
            t = t[3:].lstrip()
            kept.append(t[1:] if t.startswith("#") else t)
        elif not t.startswith("//"):
            kept.append(line)
    text = "\n".join(kept)
    out = []
    for m in re.finditer(r"(matrix|vector|vec)!\[", text):
        depth, i = 1, m.end()
        while depth:
            depth += {"[": 1, "]": -1}.get(text[i], 0)
            i += 1
        body = text[m.end():i - 1].strip()
        if m.group(1) == "matrix":
            rows = [r for r in body.split(";")] if body else []
            mat = [[_num(e) for e in r.split(",") if e.strip()] for r in rows]
            out.append(("matrix", mat))
        else:
            if ";" in body:  # vec![x; n]
                v, n = body.split(";")
                out.append(("vector", [_num(v)] * int(n)))
            else:
                out.append(("vector", [_num(e) for e in body.split(",") if e.strip()]))
    return [v for _, v in out]


def _scalars(text: str, pattern: str):
    return [float(x) for x in re.findall(pattern, text)]


def main(ref: Path) -> None:
    def span(path, lo, hi):
        lines = (ref / path).read_text().splitlines()
        return "\n".join(lines[lo - 1:hi])

    cases = {}

    def add(name, path, lo, hi, roles, **extra):
        lits = _literals(span(path, lo, hi))
        if len(lits) != len(roles):
            raise SystemExit(f"{name}: expected {len(roles)} literals at {path}:{lo}-{hi}, found {len(lits)}")
        case = {"cite": f"{path}:{lo}-{hi}"}
        case.update(dict(zip(roles, lits)))
        case.update(extra)
        cases[name] = case

    lu = "src/matrix/decomposition/lu.rs"
    ch = "src/matrix/decomposition/cholesky.rs"
    qr = "src/matrix/decomposition/qr.rs"
    hh = "src/matrix/decomposition/householder.rs"
    mm = "src/matrix/mat_mul.rs"
    im = "src/matrix/impl_mat.rs"
    tm = "tests/mat/mod.rs"
    pm = "src/matrix/permutation_matrix.rs"

    # PartialPivLu
    add("lu_exact_3x3", tm, 104, 120, ["a", "l", "u", "p"])
    add("lu_reconstruct_5x5", tm, 128, 132, ["a"])
    add("lu_reconstruct_9x9", tm, 143, 151, ["a"])
    add("lu_reconstruct_4x4_d", tm, 161, 164, ["a"])
    add("lu_reconstruct_4x4_x", lu, 781, 784, ["a"])
    add("lu_inverse_4x4", lu, 809, 817, ["a", "inv"])
    add("lu_det_4x4", lu, 836, 843, ["a"], det=_scalars(span(lu, 843, 843), r"=\s*([-0-9.eE]+);")[0])
    add("lu_solve_4x4", lu, 849, 854, ["a", "b", "x"], ulp_tol=100)
    add("lu_singular_4x4", lu, 761, 766, ["a"], error="DivByZero")
    add("lu_forward_substitution", lu, 869, 887, ["lu0", "b0", "lu1", "b1", "x1", "lu2", "b2", "x2"])
    add("solve_poisson_9x9", tm, 5, 19, ["a", "b", "x"], abs_tol=1e-8)
    # FullPivLu
    add("full_lu_reconstruct_4x4", lu, 898, 901, ["a"])
    add("full_lu_singular_rank3", lu, 916, 919, ["a"], rank=3)
    add("full_lu_solve_4x4", lu, 947, 952, ["a", "b", "x"], ulp_tol=100)
    add("full_lu_inverse_4x4", lu, 965, 973, ["a", "inv"])
    add("full_lu_noninvertible_3x3", lu, 982, 984, ["a"], error="DivByZero")
    add("full_lu_doc_rank2", lu, 537, 539, ["a"], rank=2)
    # Matrix::solve / det
    dets = _scalars(span(im, 652, 677), r"assert(?:_scalar)?_eq!\([a-z], ([-0-9.]+)")
    add("matrix_det", im, 649, 675, ["a2", "c3", "e5", "g4"], dets=dets)
    add("matrix_solve_2x2", im, 682, 685, ["a", "y"], x=[1.0, 2.0])
    add("matrix_solve_doc", im, 335, 341, ["a", "y", "x"])
    # Cholesky
    add("cholesky_unpack_1x1_2x2", ch, 394, 408, ["a1", "l1", "a2", "l2"])
    add("cholesky_fails", ch, 420, 439, ["a1", "a2", "a3", "a4"], error="DecompFailure")
    add("cholesky_det", ch, 454, 462, ["a1", "a2"], dets=[1.0, 36.0])
    add("cholesky_solve", ch, 480, 492, ["a1", "b1", "x1", "a2", "b2", "x2"])
    add("cholesky_inverse", ch, 509, 533, ["a1", "inv1", "a2", "inv2", "a3", "inv3"])
    add("cholesky_doc", ch, 46, 77, ["a", "l", "a_again", "b1", "b2", "x1", "x2"])
    add("transpose_back_substitution", ch, 568, 589, ["l1", "b1", "x1", "l2", "b2", "x2", "l3", "b3", "x3"])
    add("cholesky_legacy_3x3", tm, 176, 184, ["a", "l_flat"])
    # HouseholderQr
    shapes = _literals(span(qr, 436, 576))
    cases["qr_reconstruct_shapes"] = {"cite": f"{qr}:436-576", "mats": shapes, "ulp_tol": 100}
    add("qr_legacy_3x3", tm, 190, 201, ["a", "q", "r"], abs_tol=1e-6)
    add("householder_compute", hh, 337, 349, ["x1", "x2", "x3"])
    add("householder_left_multiply", hh, 357, 376, ["a", "v", "buffer", "expected"], tau=0.06666666666666667,
        abs_tol=1e-3)
    add("householder_composition", hh, 382, 430,
        ["storage", "tau", "x_square", "e_square", "x_tall", "e_tall", "x_short", "e_short"], eps=1e-15)
    add("householder_first_k_columns", hh, 436, 445, ["storage", "tau", "q"])
    # GEMM
    c_exp = _scalars(span(mm, 307, 315), r", ([-0-9.]+)\);")
    add("gemm_f32_3x2_2x3", mm, 295, 299, ["a", "b"], c=c_exp, dtype="f32")
    add("gemm_f64_3x2_2x3", mm, 320, 324, ["a", "b"], c=_scalars(span(mm, 332, 340), r", ([-0-9.]+)\);"))
    add("gemm_slice_uneven", mm, 400, 403, ["a", "c"], e=_scalars(span(mm, 408, 411), r", ([-0-9.]+)\);"),
        slice_of_c=[0, 0, 2, 2])
    # PermutationMatrix
    add("perm_swap_rows", pm, 526, 526, ["expected"], swaps=[[0, 3], [1, 3]], n=4)
    add("perm_parity", pm, 598, 604, ["even", "odd"])
    add("perm_inverse", pm, 590, 591, ["p", "inverse"])
    add("perm_invalid", pm, 559, 561, ["a", "b", "c"])
    (HERE / "reference_cases.json").write_text(json.dumps(cases, indent=1, sort_keys=True) + "\n")
    print(f"wrote {len(cases)} cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_golden.py <path of the rulinalg 0.4.2 source tree>")
    main(Path(sys.argv[1]))

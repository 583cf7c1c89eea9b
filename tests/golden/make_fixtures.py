"""Regenerate the golden fixtures under tests/golden/ from the reference tree.

Run in the development container, where the reference checkout is mounted
(pass its root as the first argument).  The outputs are committed; nothing
reads the reference at test time.

Outputs
-------
water_sto3g.npz
    S, T, V (7x7) and TEI (7^4) of water/STO-3G, expanded exactly as
    ``read_tensor`` does in
    ``libs/Einsums/TensorAlgebra/tests/unit/QChemTests.cpp:33-91`` (2-fold
    symmetry for matrices, 8-fold for TEI), from the fixture files
    ``libs/Einsums/TensorAlgebra/tests/unit/data/water_sto3g/{S,T,V,TEI}.dat``.
golden.json
    * ``qchem``: nuclear repulsion and the asserted SCF / MP2 / total energies
      of ``TEST_CASE("RHF No symmetry")`` (QChemTests.cpp:255, 341, 413-414).
    * ``cpp_choices``: every ``einsum(..., &alg_choice)`` call followed by an
      active ``REQUIRE(alg_choice == ...)`` in
      ``libs/Einsums/TensorAlgebra/tests/unit/*.cpp`` -- (C, A, B index
      labels, expected AlgorithmChoice, file:line).
    * ``py_plans``: every ``compile_plan(C, A, B)`` followed by
      ``assert type(plan) is ein.core.<Plan>`` in the reference's pytest suite
      (``tests/test_*.py``).
    * ``known_answers``: the exact integer results asserted in
      ``Einsum1.cpp:17-88`` (and repeated over 10 tensors in ``Batched.cpp``).
    * ``qchem_symmetry``: the symmetrizer matrix, orbitals per irrep and TEI
      tile list of ``TEST_CASE("RHF symmetry")`` (QChemTests.cpp:417).
"""
from __future__ import annotations

import glob
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_tensor(path: str, rank: int, n: int = 7) -> np.ndarray:
    out = np.zeros((n,) * rank)
    with open(path) as f:
        for line in f:
            parts = line.split()
            if not parts:
                continue
            idx = [int(p) - 1 for p in parts[:rank]]
            val = float(parts[rank])
            if rank == 2:
                i, j = idx
                out[i, j] = val
                out[j, i] = val
            else:
                i, j, k, l = idx
                for t in ((i, j, k, l), (i, j, l, k), (j, i, k, l), (j, i, l, k), (k, l, i, j),
                          (l, k, i, j), (k, l, j, i), (l, k, j, i)):
                    out[t] = val
    return out


_IDX = re.compile(r"Indices\{([^}]*)\}")


def _labels(group: str):
    return [t.strip().replace("index::", "") for t in group.split(",") if t.strip()]


def cpp_choices(unit_dir: str):
    found = []
    for path in sorted(glob.glob(os.path.join(unit_dir, "*.cpp"))):
        text = open(path).read()
        lines = text.split("\n")
        for m in re.finditer(r"einsum\(", text):
            start = m.start()
            # the call ends at the first ");" after it
            end = text.find(");", start)
            call = text[start:end]
            if "&alg_choice" not in call:
                continue
            groups = _IDX.findall(call)
            if len(groups) != 3:
                continue
            line_no = text.count("\n", 0, end) + 1
            # the assertion must be the next non-empty statement and not commented
            nxt = None
            for k in range(line_no, min(line_no + 3, len(lines))):
                s = lines[k].strip()
                if s:
                    nxt = s
                    break
            if nxt is None or not nxt.startswith("REQUIRE(alg_choice =="):
                continue
            choice = re.search(r"detail::(\w+)\)", nxt).group(1)
            found.append({"C": _labels(groups[0]), "A": _labels(groups[1]), "B": _labels(groups[2]),
                          "expected": choice,
                          "where": f"libs/Einsums/TensorAlgebra/tests/unit/{os.path.basename(path)}:{line_no + 1}"})
    return found


def py_plans(tests_dir: str):
    found = []
    for path in sorted(glob.glob(os.path.join(tests_dir, "test_*.py"))):
        lines = open(path).read().split("\n")
        for i, line in enumerate(lines):
            m = re.search(r'compile_plan\("([^"]*)",\s*"([^"]*)",\s*"([^"]*)"\)', line)
            if not m:
                continue
            for k in range(i + 1, min(i + 4, len(lines))):
                t = re.search(r"assert type\(plan\) is ein\.core\.(\w+)", lines[k])
                if t:
                    found.append({"C": m.group(1), "A": m.group(2), "B": m.group(3),
                                  "expected": t.group(1),
                                  "where": f"tests/{os.path.basename(path)}:{i + 1}"})
                    break
    # deduplicate, keeping the first location
    seen, out = set(), []
    for f in found:
        key = (f["C"], f["A"], f["B"], f["expected"])
        if key not in seen:
            seen.add(key)
            out.append(f)
    return out


def known_answers(unit_dir: str):
    text = open(os.path.join(unit_dir, "Einsum1.cpp")).read()
    sections = []
    for sec in re.finditer(r'SECTION\("([^"]+)"\)', text):
        body = text[sec.end(): text.find("SECTION(", sec.end()) if text.find("SECTION(", sec.end()) > 0 else None]
        vals = re.findall(r"REQUIRE\(C\((\d), (\d)\) == ([0-9.]+)\);", body)
        if vals:
            sections.append({"section": sec.group(1),
                             "values": [[int(i), int(j), float(v)] for i, j, v in vals]})
    return sections


def qchem(unit_dir: str):
    text = open(os.path.join(unit_dir, "QChemTests.cpp")).read()
    enuc = float(re.search(r"double enuc = ([0-9.]+);", text).group(1))
    e_scf = float(re.search(r"REQUIRE_THAT\(e0, Catch::Matchers::WithinAbs\(([-0-9.]+), 1e-6\)\)", text).group(1))
    e_mp2 = float(re.search(r"REQUIRE_THAT\(eMP2, Catch::Matchers::WithinAbs\(([-0-9.]+), 1e-6\)\)", text).group(1))
    e_tot = float(re.search(r"REQUIRE_THAT\(e_tot, Catch::Matchers::WithinAbs\(([-0-9.]+), 1e-6\)\)", text).group(1))
    return {"enuc": enuc, "e_scf": e_scf, "e_mp2": e_mp2, "e_tot": e_tot, "tol": 1e-6,
            "where": "libs/Einsums/TensorAlgebra/tests/unit/QChemTests.cpp:185-415"}


def qchem_symmetry(unit_dir: str):
    """The symmetry-adapted inputs of TEST_CASE("RHF symmetry") (QChemTests.cpp:417-...): the
    7x7 matrix that forms the C2v symmetry-adapted combinations (``symm_values``), the orbitals
    per irrep (``irrep_sizes``) and the TEI tiles the test fills (``TEI_sym.tile(...) = ...``)."""
    text = open(os.path.join(unit_dir, "QChemTests.cpp")).read()
    start = text.index('TEST_CASE("RHF symmetry")')
    body = text[start:]
    vals = re.search(r"std::vector<double>\s+symm_values\{([^}]*)\}", body).group(1)
    symm = []
    for tok in vals.replace("\n", " ").split(","):
        tok = tok.strip()
        neg = tok.startswith("-")
        tok = tok.lstrip("-")
        v = 1.0 / np.sqrt(2.0) if tok == "M_SQRT1_2" else float(tok)
        symm.append(-v if neg else v)
    sizes = [int(x) for x in re.search(r"irrep_sizes\{([^}]*)\}", body).group(1).split(",")]
    tiles = [[int(x) for x in m.group(1).split(",")] for m in re.finditer(r"TEI_sym\.tile\(([0-9, ]+)\)\s*=", body)]
    line = text.count("\n", 0, start) + 1
    return {"symm": symm, "irrep_sizes": sizes, "tei_tiles": tiles,
            "where": f"libs/Einsums/TensorAlgebra/tests/unit/QChemTests.cpp:{line}"}


def main(ref_root: str):
    unit = os.path.join(ref_root, "libs/Einsums/TensorAlgebra/tests/unit")
    data = os.path.join(unit, "data/water_sto3g")
    np.savez_compressed(os.path.join(HERE, "water_sto3g.npz"),
                        S=read_tensor(os.path.join(data, "S.dat"), 2),
                        T=read_tensor(os.path.join(data, "T.dat"), 2),
                        V=read_tensor(os.path.join(data, "V.dat"), 2),
                        TEI=read_tensor(os.path.join(data, "TEI.dat"), 4))
    golden = {"qchem": qchem(unit), "cpp_choices": cpp_choices(unit),
              "py_plans": py_plans(os.path.join(ref_root, "tests")),
              "known_answers": known_answers(unit), "qchem_symmetry": qchem_symmetry(unit)}
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    print(f"cpp_choices={len(golden['cpp_choices'])} py_plans={len(golden['py_plans'])} "
          f"known_answers={len(golden['known_answers'])}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")

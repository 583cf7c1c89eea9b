"""Water/STO-3G RHF + MP2, written as the reference's golden physics test.

Restates ``TEST_CASE("RHF No symmetry")`` of
``libs/Einsums/TensorAlgebra/tests/unit/QChemTests.cpp:185-415`` call for
call: every contraction goes through the ``einsum`` callable under test, with
the same index patterns (the Fock build uses the GEMV pattern
``ij <- kl * ijkl`` and the GENERIC pattern ``ij <- kl * ikjl``).  The
diagonalisations (``syev``, ``pow(S, -0.5)``) are not on the einsum path and
run in numpy.

``ops`` adapts the driver to an array backend:
    ops.einsum(C_labels, C, c_pref, ab_pref, A_labels, A, B_labels, B)
    ops.array(np.ndarray) -> backend array (a copy)
    ops.numpy(backend array) -> np.ndarray
    ops.zeros(shape) -> backend array
    ops.scalar(backend rank-0 array) -> float
    ops.copy_into(dst, src) (dst[...] = src)
    ops.fock(F, TEI, D) (optional: F += 2 J - K in one call)
"""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_water():
    z = np.load(os.path.join(GOLDEN, "water_sto3g.npz"))
    return {k: z[k].copy() for k in ("S", "T", "V", "TEI")}


def _inv_sqrt(S):
    w, U = np.linalg.eigh(S)
    return (U * w ** -0.5) @ U.T


def rhf_mp2(ops, enuc: float, max_cycles: int = 50):
    w = load_water()
    n, nocc = 7, 5
    H_np = w["T"] + w["V"]
    X_np = _inv_sqrt(w["S"])
    H, X = ops.array(H_np), ops.array(X_np)
    TEI = ops.array(w["TEI"])
    F = ops.array(H_np)
    temp1, Ft, C, D = ops.zeros((n, n)), ops.zeros((n, n)), ops.zeros((n, n)), ops.zeros((n, n))
    Elec = ops.zeros(())

    def transform_and_diag():
        ops.einsum("ij", temp1, 0.0, 1.0, "ik", F, "kj", X)
        ops.einsum("ij", Ft, 0.0, 1.0, "kj", temp1, "ki", X)
        evals, Ct_np = np.linalg.eigh(ops.numpy(Ft))
        Ct = ops.array(Ct_np)
        ops.einsum("ij", C, 0.0, 1.0, "kj", Ct, "ik", X)
        Cocc = C[:, 0:nocc]
        ops.einsum("ij", D, 0.0, 1.0, "im", Cocc, "jm", Cocc)
        return evals

    def energy():
        ops.copy_into(Elec, np.zeros(()))
        ops.einsum("", Elec, 0.0, 1.0, "ij", D, "ij", F)
        ops.einsum("", Elec, 1.0, 1.0, "ij", D, "ij", H)
        return ops.scalar(Elec) + enuc

    evals = transform_and_diag()
    e0, e1, drms, cycles = energy(), 0.0, 1.0, 0
    while abs(e0 - e1) > 1e-10 and drms > 1e-6 and cycles < max_cycles:
        cycles += 1
        e1 = e0
        D_prev = ops.numpy(D).copy()
        ops.copy_into(F, H_np)
        if hasattr(ops, "fock"):
            ops.fock(F, TEI, D)  # F += 2 J - K through a symmetric-integral entry point
        else:
            ops.einsum("ij", F, 1.0, 2.0, "kl", D, "ijkl", TEI)
            ops.einsum("ij", F, 1.0, -1.0, "kl", D, "ikjl", TEI)
        evals = transform_and_diag()
        e0 = energy()
        diff = ops.array(ops.numpy(D) - D_prev)
        rms = ops.zeros(())
        ops.einsum("", rms, 0.0, 1.0, "ij", diff, "ij", diff)
        drms = float(np.sqrt(ops.scalar(rms)) / 7.0)

    # MP2: transform the integrals to the MO basis (QChemTests.cpp:349-356).
    t1, t2 = ops.zeros((n,) * 4), ops.zeros((n,) * 4)
    ops.einsum("pqrs", t1, 0.0, 1.0, "mqrs", TEI, "mp", C)
    ops.einsum("pqrs", t2, 0.0, 1.0, "pmrs", t1, "mq", C)
    ops.einsum("pqrs", t1, 0.0, 1.0, "pqms", t2, "mr", C)
    ops.einsum("pqrs", TEI, 0.0, 1.0, "pqrm", t1, "ms", C)
    e = evals
    scale = 1.0 / (e[:nocc, None, None, None] + e[None, None, :nocc, None]
                   - e[None, nocc:, None, None] - e[None, None, None, nocc:])
    scale_b = ops.array(scale)
    tei_iajb = TEI[0:nocc, nocc:n, 0:nocc, nocc:n]
    amps = ops.zeros((nocc, n - nocc, nocc, n - nocc))
    ops.einsum("iajb", amps, 0.0, 1.0, "iajb", tei_iajb, "iajb", scale_b)
    e_a, e_b = ops.zeros(()), ops.zeros(())
    ops.einsum("", e_a, 0.0, 2.0, "iajb", amps, "iajb", tei_iajb)
    ops.einsum("", e_b, 0.0, -1.0, "iajb", amps, "ibja", tei_iajb)
    emp2 = ops.scalar(e_a) + ops.scalar(e_b)
    return {"e_scf": e0, "e_mp2": emp2, "e_tot": e0 + emp2, "cycles": cycles}

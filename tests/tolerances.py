"""The value tolerance of every Generate parity test.

A matrix entry A_ij is a sum over elements of entries of element matrices,
each itself a sum over Gauss points of products.  The GPU adds the element
contributions in another order (FP64 atomics) and evaluates each with fused
multiply-adds and algebraically equal formulas, so it differs from the
reference by rounding, whose scale is not |A_ij|: many entries are residues
of cancellation (about 20 % of the P2 elasticity entries on the Kuhn mesh are
below 1e-12 of their row's largest entry; some are zero in exact arithmetic).

Every element matrix of these formulations is symmetric positive
semi-definite (stiffness, curl-curl, mass, and the Newton Jacobian of a
monotone B-H law), so by Cauchy-Schwarz each element's contribution to
A_ij, and the rounding of its Gauss sum, is bounded by a multiple of
sqrt(A_e,ii A_e,jj), and summed over the elements by sqrt(A_ii A_jj).  The
bound per entry is therefore

    |gpu - ref| <= 1e-12 |ref| + 1e-13 S,   S = max(sqrt(D_i D_j), sum |t_k|)

with D_i = |A_ii| (for a complex system in real form, the magnitude of the
unknown's 2 x 2 diagonal block, |A_ii| + |A_i,i^1|) and sum |t_k| the
entry's sum of |element contribution| from the oracle's element loop.  It
means: entries agree to 1e-12 relative, or to 1e-13 of the Jacobi-scaled
matrix D^-1/2 A D^-1/2 that the solvers iterate on.  RHS entries use the
oracle's first-order rounding scale of the row (oracle.assemble(...,
with_abs=True)): the sum of |element contribution|, for an eliminated fixed
value |g_j| sqrt(Ek_ii Ek_jj), and for the nonlinear terms evaluated at a
field b = sum_i a_i curl N_i the field's own rounding (the nodal values
cancel in the curl) times the B-H law's sensitivity 1 + 2 |b|^2 / b_sat^2;
1e-13 is about 450 units in the last place of that scale.
"""
import numpy as np

VAL_REL = 1e-12
SUM_REL = 1e-13


def diag_scale(indptr, indices, data, complex_pairs=False):
    """Per entry, sqrt(D_row D_col) from the reference matrix's diagonal."""
    indptr = np.asarray(indptr, np.int64)
    indices = np.asarray(indices, np.int64)
    n = len(indptr) - 1
    rows = np.repeat(np.arange(n), np.diff(indptr))
    ad = np.abs(np.asarray(data, np.float64))
    D = np.zeros(n)
    on = indices == rows
    np.add.at(D, rows[on], ad[on])
    if complex_pairs:
        partner = indices == (rows ^ 1)
        np.add.at(D, rows[partner], ad[partner])
    return np.sqrt(D[rows] * D[indices])


def bound(ref, scale):
    return VAL_REL * np.abs(ref) + SUM_REL * np.asarray(scale)


def values_close(got, ref, scale):
    return bool(np.all(np.abs(got - ref) <= bound(ref, scale)))


def matrix_scale(indptr, indices, data, abs_sum, complex_pairs=False):
    """S of the matrix entries: the larger of the diagonal scale and the
    sum of |element contribution|."""
    return np.maximum(diag_scale(indptr, indices, data, complex_pairs), abs_sum)


def report(got, ref, scale):
    """(worst ratio |gpu - ref| / bound, entries beyond 1e-12 relative)."""
    d = np.abs(got - ref)
    ratio = d / np.maximum(bound(ref, scale), 1e-300)
    return float(ratio.max(initial=0.0)), int(np.sum(d > VAL_REL * np.abs(ref)))

"""Post-processing (PostOperation Print[ {d a}, OnElementsOf ], Print[ {a},
OnPoint ], Print[ {d a}, OnPoint ]) against the reference's printed values
(tests/golden/post_*.npz, made by make_post_golden.py) and the oracle.

Tolerance: 1e-13 relative to the field's magnitude; for the curl of the
edge-element field the bound is 1e-13 * sum_e |a_e| |curl w_e| per element
(the curl-curl solution carries a large gradient part that cancels in the
curl, so the sum's own condition sets the attainable accuracy).
"""
import numpy as np
import pytest

from getdp_gb300 import workloads as W
from oracle import post_port as PP
from tests.golden_cases import GOLDEN

CASES = {"post_ms2d_n8": W.magnetostatics_2d, "post_eddy_n8": W.eddy_2d,
         "post_cc_edge_n4": W.curlcurl_edge,
         # fixed DOFs with non-zero values enter {a} and {d a}
         "post_ms2d_n8_dir": W.magnetostatics_2d, "post_eddy_n8_dir": W.eddy_2d}


def load(name):
    import os
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    kw = {str(k): (float(v) if k == "freq" else int(v))
          for k, v in zip(d["gen_kw_keys"], d["gen_kw_vals"])}
    p = CASES[name](**kw)
    return d, p, W.dofmap_for(p)


def reference_values(d, p):
    """(element curls, point fields, point curls) in the layouts of
    curl_on_elements / at_points."""
    ev, k = d["elem_vals"], d["elem_index"]
    if p.formulation == "curlcurl":
        return k, ev[:, 0, 0, :], d["pts_a"][:, 0, :], d["pts_b"][:, 0, :]
    return k, ev[:, :, 0, :2], d["pts_a"][:, :, 2], d["pts_b"][:, :, :2]


def curl_bound(p, dm, x):
    """Per element sum_e |a_e| |curl w_e| (3D) or max |a| |curl N| (2D)."""
    nodes, el = p.mesh.nodes, p.mesh.elems
    if p.formulation == "curlcurl":
        P = nodes[el]
        J = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=1)
        D = np.linalg.det(J)
        cu = np.einsum("ic,erc->eir", PP.CURL_EDGE, J.transpose(0, 2, 1)) / D[:, None, None]
        a = np.where(dm.elem_dofs >= 0, x[np.maximum(dm.elem_dofs, 0)], 0.0)
        return np.einsum("ei,ei->e", np.abs(a), np.linalg.norm(cu, axis=2))
    return None


def check_curls(p, dm, x, got, ref):
    if p.formulation == "curlcurl":
        bound = 1e-13 * curl_bound(p, dm, x)[:, None] + 1e-300
        assert np.all(np.abs(got - ref) <= bound)
    else:
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_post(name):
    d, p, dm = load(name)
    k, rb, ra, rpb = reference_values(d, p)
    b = PP.curl_on_elements(p, dm, d["x"])
    check_curls(p, dm, d["x"], b[k], rb)
    fa, fb, fe = PP.at_points(p, dm, d["x"], d["pts"])
    assert np.array_equal(fe, d["pts_elem"])
    assert np.abs(fa - ra).max() <= 1e-13 * np.abs(ra).max()
    if p.formulation == "curlcurl":
        bound = 1e-13 * curl_bound(p, dm, d["x"])[fe][:, None]
        assert np.all(np.abs(fb - rpb) <= bound)
    else:
        check_curls(p, dm, d["x"], fb, rpb)


# ----------------------------------------------------------------- GPU
def _gpu(p, dm, x, pts):
    from getdp_gb300 import build
    build.build()
    from getdp_gb300 import generate as G_
    from getdp_gb300 import linalg as LA
    from getdp_gb300 import post
    terms = G_.DeviceTerms(p, dm)
    xv = LA.gVector(dm.n_dof)
    xv.set(x)
    b = post.curl_on_elements(terms.batch, xv)
    fa, fb, fe = post.at_points(terms.batch, xv, pts)
    return b, fa, fb, fe


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_post_matches_reference(name):
    d, p, dm = load(name)
    k, rb, ra, rpb = reference_values(d, p)
    b, fa, fb, fe = _gpu(p, dm, d["x"], d["pts"])
    check_curls(p, dm, d["x"], b[k], rb)
    assert np.array_equal(fe, d["pts_elem"])
    assert np.abs(fa - ra).max() <= 1e-13 * np.abs(ra).max()
    if p.formulation == "curlcurl":
        bound = 1e-13 * curl_bound(p, dm, d["x"])[fe][:, None]
        assert np.all(np.abs(fb - rpb) <= bound)
    else:
        assert np.abs(fb - rpb).max() <= 1e-13 * np.abs(rpb).max()


@pytest.mark.gpu
@pytest.mark.parametrize("gen,n", [(W.magnetostatics_2d, 40), (W.eddy_2d, 24),
                                   (W.curlcurl_edge, 8)])
def test_gpu_post_matches_oracle_larger(gen, n):
    p = gen(n=n)
    dm = W.dofmap_for(p)
    rng = np.random.default_rng(n)
    x = rng.standard_normal(dm.n_dof)
    pts = rng.uniform(0.01, 0.99, size=(500, 3))
    if p.formulation != "curlcurl":
        pts[:, 2] = 0.0
    b, fa, fb, fe = _gpu(p, dm, x, pts)
    ob = PP.curl_on_elements(p, dm, x)
    ofa, ofb, ofe = PP.at_points(p, dm, x, pts)
    assert np.array_equal(fe, ofe)
    assert np.abs(b - ob).max() <= 1e-12 * np.abs(ob).max()
    assert np.abs(fa - ofa).max() <= 1e-12 * np.abs(ofa).max()
    assert np.abs(fb - ofb).max() <= 1e-12 * np.abs(ofb).max()


@pytest.mark.gpu
def test_gpu_post_point_outside_and_unsupported_kind():
    p = W.magnetostatics_2d(n=6)
    dm = W.dofmap_for(p)
    x = np.ones(dm.n_dof)
    b, fa, fb, fe = _gpu(p, dm, x, np.array([[1.5, 0.5, 0.0], [0.5, 0.5, 0.0]]))
    assert fe[0] == -1 and fa[0, 0] == 0.0 and fe[1] >= 0
    from getdp_gb300 import generate as G_
    from getdp_gb300 import linalg as LA
    from getdp_gb300 import post
    pe = W.elasticity_p2(n=2)
    dme = W.dofmap_for(pe)
    with pytest.raises(ValueError):
        post.curl_on_elements(G_.DeviceTerms(pe, dme).batch, LA.gVector(dme.n_dof))

"""The salt-body workload at reduced resolution (the same 8-bump body on a
43 x 136 x 136 grid, 100 m nominal spacing): the neural SDF form meshes it
like the exact isosurface SDF form, and the network's values agree with the
exact distances outside the band.

Tolerances: the exact SDF decides every value within the band and every
point that may lie outside, so generate_mesh gives the same mesh in both
forms: equal vertex and cell counts, mean quality within 1e-6.  After
sliver_removal (whose cell order, and so its tie rule between slivers that
share a vertex, follows the order in which the filter appended the cells)
the counts and mean quality agree within 1 %.  Every network value outside
the band has the sign of the exact distance."""
import contextlib
import io

import numpy as np
import pytest
import torch

import seismicmesh_gb300 as sm
from seismicmesh_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def salt(cuda):
    vp, B, bbox = S.salt_model_3d(shape=(43, 136, 136))
    with contextlib.redirect_stdout(io.StringIO()):
        ef = sm.get_sizing_function_from_segy(None, bbox, velocity_data=vp, nz=43, nx=136, ny=136,
                                              hmin=75.0, wl=10, freq=2.0, grade=0.15)
    iso = sm.Isosurface(B, bbox, 0.5)
    nn = sm.NeuralSDF(iso, 75.0, n_samples=1_000_000, epochs=40)
    return iso, nn, ef


def test_network_sign_outside_the_band(salt):
    iso, nn, ef = salt
    assert np.isfinite(nn.band) and nn.band < nn.clamp
    assert nn.stats["sign_agreement_outside_band"] == 1.0
    rng = np.random.default_rng(0)
    lo, hi = np.array(iso.bbox[0::2]), np.array(iso.bbox[1::2])
    x = lo + (hi - lo) * rng.uniform(size=(20000, 3))
    d = iso.eval(x)
    y = nn.eval_network(x)
    out = np.abs(y) >= nn.band
    assert np.all(np.sign(y[out]) == np.sign(d[out]))
    # the combined evaluation is exact wherever |value| < band
    z = nn.eval(x)
    inb = np.abs(z) < nn.band
    np.testing.assert_allclose(z[inb], d[inb], rtol=0, atol=1e-3)


def test_neural_and_exact_forms_give_the_same_mesh(salt):
    from oracle import mesh_qa_np as QA

    iso, nn, ef = salt
    gen, sl = {}, {}
    for name, dom in (("exact", iso), ("neural", nn)):
        p, t = sm.generate_mesh(dom, ef, verbose=0)
        q, _ = QA.cell_quality_vec(p, t)
        gen[name] = (len(p), len(t), float(q.mean()))
        p2, t2 = sm.sliver_removal(p, dom, ef, verbose=0)
        q2, _ = QA.cell_quality_vec(p2, t2)
        sl[name] = (len(p2), len(t2), float(q2.mean()))
        print(name, gen[name], sl[name])
    assert gen["neural"][:2] == gen["exact"][:2]
    assert abs(gen["neural"][2] - gen["exact"][2]) <= 1e-6
    assert sl["neural"][0] == sl["exact"][0]
    assert abs(sl["neural"][1] - sl["exact"][1]) <= 0.01 * sl["exact"][1]
    assert abs(sl["neural"][2] - sl["exact"][2]) <= 0.01 * sl["exact"][2]

"""Driver-script text formats (run/fastpm/fastpm.py:95-103, :150-166) and the
ijl triangle ordering (util.py:8-24).  CPU only."""
import numpy as np

from pyspectrum_gb300 import core, outputs, util


def _fake_bispec(T=40, seed=0):
    rng = np.random.default_rng(seed)
    tri = core.triangles(1, 6)[:, :T]
    b = {"i_k1": tri[0] * 3, "i_k2": tri[1] * 3, "i_k3": tri[2] * 3}
    for k in ("p0k1", "p0k2", "p0k3", "b123", "q123", "counts", "b123_sn"):
        b[k] = rng.normal(size=tri.shape[1]) * 1e4
    return b


def test_bk_table_roundtrip_and_header(tmp_path):
    b = _fake_bispec()
    p = tmp_path / "bk.dat"
    outputs.save_bk(p, b, 2500.0)
    lines = p.read_text().splitlines()
    assert lines[0] == "# pyspectrum bispectrum calculation test. k_f = 2pi/2500.0"
    assert lines[1] == "#  i_k1, i_k2, i_k3, p0k1, p0k2, p0k3, bk, qk, counts, bk_shotnoise"
    assert len(lines[2].split()) == 10 and lines[2].split()[0] == str(b["i_k1"][0])
    back = outputs.load_bk(p)
    for k in outputs.BK_COLUMNS:
        np.testing.assert_allclose(back[k], b[k], rtol=1e-5)


def test_bk_table_in_ijl_order(tmp_path):
    b = _fake_bispec()
    order = util.ijl_order(b["i_k1"], b["i_k2"], b["i_k3"], typ="GM")
    p = tmp_path / "bk.dat"
    outputs.save_bk(p, b, 2500.0, order=order)
    back = outputs.load_bk(p)
    key = back["i_k3"] * 10 ** 6 + back["i_k2"] * 10 ** 3 + back["i_k1"]
    assert np.all(np.diff(key) > 0)          # sorted by l, then j, then i


def test_pk_table_roundtrip_and_header(tmp_path):
    k = np.linspace(0.01, 0.5, 30)
    pk = 1e4 / (1 + (k / 0.1) ** 2)
    cnt = np.arange(30) * 10.0 + 4
    p = tmp_path / "pk.dat"
    outputs.save_pk(p, k, pk, cnt, Nhalo=73442, Lbox=2600.0, kf=2 * np.pi / 2600.0, nbar=73442 / 2600.0 ** 3)
    lines = p.read_text().splitlines()
    assert lines[0].startswith("# pySpectrum P_l=0(k). Nhalo=73442, Lbox=2600, k_f=2.41661e-03, SN=")
    assert lines[1] == "#  k, p0k, counts"
    kk, pp, cc = outputs.load_pk(p)
    np.testing.assert_allclose(kk, k, rtol=1e-5)
    np.testing.assert_allclose(pp, pk, rtol=1e-5)
    np.testing.assert_array_equal(cc, cnt)

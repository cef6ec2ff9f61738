"""GPU lattice build (Permutohedral::init on the device) against the reference's
golden tables and the oracle: bit-exact offsets, ranks, barycentric weights,
neighbours and keys -- vertex ids included, no relabelling."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VARIANTS = (("sse", 0), ("scalar", 1))


def _bits(a):
    return np.ascontiguousarray(a).view(np.int32)


def _gpu_lattice(dc, feat_nd, variant, M=2):
    N, d = feat_nd.shape
    crf = dc.DenseCRF(N, M)
    crf.set_variant(variant)
    crf.addPairwiseEnergy(np.ascontiguousarray(feat_nd.T), compat=1.0)
    return crf.lattice(0)


@pytest.mark.parametrize("vname,var", VARIANTS)
def test_lattice_matches_reference_golden(engine, golden, vname, var):
    g = golden("lattice.npz")
    names = sorted({k.split("/")[0] for k in g.files})
    for name in names:
        lat = _gpu_lattice(engine, g[f"{name}/feat"], var)
        assert np.array_equal(lat["offset"], g[f"{name}/{vname}/offset"]), name
        assert np.array_equal(lat["rank"], g[f"{name}/{vname}/rank"]), name
        assert np.array_equal(_bits(lat["bary"]), _bits(g[f"{name}/{vname}/bary"])), name
        assert np.array_equal(lat["neighbors"], g[f"{name}/{vname}/neighbors"]), name


@pytest.mark.parametrize("vname,var", VARIANTS)
def test_lattice_matches_oracle_random(engine, oracle_mod, vname, var):
    rng = np.random.default_rng(5 + var)
    for d in (1, 2, 3, 4, 5, 6, 7, 8, 11, 16):
        for N in (1, 2, 3, 4, 5, 255, 256, 257, 1000, 4099):
            f = rng.normal(0, 2.0 + d, size=(N, d)).astype(np.float32)
            lat = _gpu_lattice(engine, f, var)
            ref = oracle_mod.Lattice(f, "oracle", var)
            assert lat["L"] == ref.L, (d, N)
            assert np.array_equal(lat["offset"], ref.offset), (d, N)
            assert np.array_equal(lat["rank"], ref.rank), (d, N)
            assert np.array_equal(_bits(lat["bary"]), _bits(ref.bary)), (d, N)
            assert np.array_equal(lat["neighbors"], ref.neighbors), (d, N)
            assert np.array_equal(lat["keys"], ref.keys), (d, N)


def test_lattice_image_features(engine, oracle_mod):
    """2D and bilateral image features (integer-valued positions: rounding ties)."""
    from pydensecrf_gb300 import synthetic as S
    cfg = S.plain_small(1)
    O = oracle_mod
    for f in (O.features_gaussian_2d(320, 240, 3.0, 3.0), O.features_bilateral_2d(cfg["img"], 80, 80, 13, 13, 13),
              O.features_gaussian_2d(37, 23, 1.0, 1.0)):
        for var in (0, 1):
            lat = _gpu_lattice(engine, f, var)
            ref = O.Lattice(f, "oracle", var)
            assert np.array_equal(lat["offset"], ref.offset)
            assert np.array_equal(_bits(lat["bary"]), _bits(ref.bary))
            assert np.array_equal(lat["neighbors"], ref.neighbors)


def test_lattice_2d_handle_equals_generic(engine, oracle_mod):
    """DenseCRF2D builds the features on the device; tables equal the host-built ones."""
    from pydensecrf_gb300 import synthetic as S
    cfg = S.plain_small(2, W=61, H=43)
    d2 = engine.DenseCRF2D(61, 43, 5)
    d2.addPairwiseGaussian(3, 3)
    d2.addPairwiseBilateral(80, 13, cfg["img"], 10)
    O = oracle_mod
    for k, f in enumerate((O.features_gaussian_2d(61, 43, 3, 3), O.features_bilateral_2d(cfg["img"], 80, 80, 13, 13, 13))):
        lat = d2.lattice(k)
        ref = O.Lattice(f, "oracle", 0)
        assert np.array_equal(lat["offset"], ref.offset)
        assert np.array_equal(_bits(lat["bary"]), _bits(ref.bary))
        assert np.array_equal(lat["neighbors"], ref.neighbors)


def test_key_overflow_is_an_error(engine):
    """Coordinates beyond the reference's int16 keys are reported, not wrapped."""
    N = 16
    f = np.zeros((N, 2), np.float32)
    f[:, 0] = np.linspace(0, 1e6, N)
    crf = engine.DenseCRF(N, 2)
    with pytest.raises(ValueError, match="int16"):
        crf.addPairwiseEnergy(np.ascontiguousarray(f.T), compat=1.0)
    # the handle stays usable
    crf.addPairwiseEnergy(np.ascontiguousarray((f / 1e5).T), compat=1.0)

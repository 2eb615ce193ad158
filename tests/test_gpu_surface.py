"""Greek surfaces on the GPU (kx_greek_surface): every cell equals
kx_greeks_bump at that cell bit for bit (one launch values all cells on the
same normals, as the reference reprices each cell on the same seed), the
FP64 surface matches the oracle's greek_surface, and the reference's own
checks (tests/surface.rs) hold on the engine."""
import math

import pytest

import kontracts_gb300 as kx

pytestmark = pytest.mark.gpu

R = 0.05
FIELDS = kx.GreekSurface.QUANTITIES


def _bs_delta_vega(s, k, r, sigma, t):
    d1 = (math.log(s / k) + (r + 0.5 * sigma * sigma) * t) / (sigma * math.sqrt(t))
    nd1 = 0.5 * (1.0 + math.erf(d1 / math.sqrt(2.0)))
    pdf = math.exp(-0.5 * d1 * d1) / math.sqrt(2.0 * math.pi)
    return nd1, s * pdf * math.sqrt(t)


CONTRACTS = {
    "call": lambda: kx.european_call("X", 100.0, 1.0),
    "up_and_out": lambda: kx.up_and_out_call("X", 100.0, 130.0, 1.0),
    "asian": lambda: kx.scale((kx.average(kx.S("X")) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0),
}


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("name", sorted(CONTRACTS))
@pytest.mark.parametrize("relative", [False, True])
def test_cells_equal_single_greeks(name, prec, relative):
    c = CONTRACTS[name]()
    spots, vols = [85.0, 100.0, 115.0], [0.15, 0.3]
    bumps = (1e-2, 1e-2, 1e-3) if relative else (0.5, 1e-2, 1e-4)
    s = kx.greek_surface(c, "X", spots, vols, n_paths=30_000, seed=11, steps_per_year=52, rate=R, bumps=bumps,
                         relative=relative, precision=prec)
    for i, sp in enumerate(spots):
        for j, v in enumerate(vols):
            g = c.greeks(kx.GBM(s0=sp, sigma=v, r=R, asset="X"), n_paths=30_000, seed=11, steps_per_year=52,
                         bumps=bumps, relative=relative, precision=prec)
            for q in FIELDS:
                assert getattr(s, q)[i, j] == getattr(g, q), (name, sp, v, q)


@pytest.mark.parametrize("name", ["call", "up_and_out"])
def test_fp64_surface_matches_oracle(orc, name):
    c = CONTRACTS[name]()
    spots, vols = [90.0, 100.0, 110.0], [0.2, 0.35]
    hs, hv, hr = 1e-2, 1e-2, 1e-4
    s = kx.greek_surface(c, "X", spots, vols, n_paths=20_000, seed=5, steps_per_year=50, rate=R, precision="fp64")
    ref = orc.greek_surface(c.to_json(), "X", spots, vols, n_paths=20_000, seed=5, steps_per_year=50, rate=R)
    for i in range(len(spots)):
        for j in range(len(vols)):
            r = ref[i * len(vols) + j]
            # the engine averages per-path differences, the reference differences
            # of averages: equal up to the rounding of a mean over the bump size
            scale = {"price": 1.0, "delta": 1 / hs, "gamma": 1 / hs ** 2, "vega": 1 / hv, "rho": 1 / hr}
            for q, k in scale.items():
                tol = 1e-9 * max(1.0, abs(r[q])) + 1e-12 * abs(r["price"]) * k
                assert abs(getattr(s, q)[i, j] - r[q]) <= tol, (name, i, j, q, getattr(s, q)[i, j], r[q])


def test_delta_and_vega_surfaces_match_black_scholes():
    """tests/surface.rs:78-113: delta within 2 %, vega within 3 % of
    Black-Scholes at every cell (spot bump 1, 200,000 paths, seed 2024)."""
    spots, vols = [90.0, 100.0, 110.0], [0.15, 0.20, 0.25]
    s = kx.greek_surface(kx.european_call("AAPL", 100.0, 1.0), "AAPL", spots, vols, n_paths=200_000, seed=2024,
                         steps_per_year=1, rate=R, bumps=(1.0, 1e-2, 1e-4))
    assert s.delta.shape == s.gamma.shape == s.vega.shape == s.price.shape == (3, 3)
    for i, sp in enumerate(spots):
        for j, v in enumerate(vols):
            d_bs, v_bs = _bs_delta_vega(sp, 100.0, R, v, 1.0)
            assert abs(s.delta[i, j] - d_bs) / d_bs < 0.02
            assert abs(s.vega[i, j] - v_bs) / v_bs < 0.03


def test_delta_increases_with_spot_and_exports():
    """tests/surface.rs:115-153."""
    s = kx.greek_surface(kx.european_call("AAPL", 100.0, 1.0), "AAPL", [80.0, 100.0, 120.0], [0.20],
                         n_paths=200_000, seed=2024, steps_per_year=1, rate=R)
    assert s.delta[0, 0] < s.delta[1, 0] < s.delta[2, 0]
    s = kx.greek_surface(kx.european_call("AAPL", 100.0, 1.0), "AAPL", [95.0, 105.0], [0.18, 0.22],
                         n_paths=200_000, seed=2024, steps_per_year=1, rate=R)
    csv = s.to_csv(s.delta)
    assert csv.startswith("spot\\vol,0.18,0.22") and len(csv.splitlines()) == 3
    assert s.to_pgm(s.delta).startswith("P2\n2 2\n255")


def test_large_grid_many_contracts_in_one_launch():
    """A 12 x 10 grid of a barrier option: 120 cells of seven scenarios each in
    one path launch; corner and centre cells equal single-cell Greeks."""
    c = CONTRACTS["up_and_out"]()
    spots = [80.0 + 4.0 * i for i in range(12)]
    vols = [0.1 + 0.03 * j for j in range(10)]
    s = kx.greek_surface(c, "X", spots, vols, n_paths=8_000, seed=3, steps_per_year=100, rate=R)
    assert kx.last_launch_stats()["kernel_launches"] >= 1
    for i, j in ((0, 0), (11, 9), (6, 4), (0, 9)):
        g = c.greeks(kx.GBM(s0=spots[i], sigma=vols[j], r=R, asset="X"), n_paths=8_000, seed=3, steps_per_year=100)
        for q in FIELDS:
            assert getattr(s, q)[i, j] == getattr(g, q), (i, j, q)


def test_rejections():
    c = CONTRACTS["call"]()
    for spots, vols in (([], [0.2]), ([100.0], [])):
        with pytest.raises(kx.KontractError) as e:
            kx.greek_surface(c, "X", spots, vols, n_paths=100)
        assert e.value.status == "InconsistentPath"
    with pytest.raises(kx.KontractError) as e:
        kx.greek_surface(c, "X", [100.0], [0.2, 0.005], n_paths=100)  # vol bump 0.01 > 0.005
    assert e.value.status == "MalformedContract"
    with pytest.raises(kx.KontractError) as e:
        kx.greek_surface(c, "X", [100.0], [0.2], n_paths=100, bumps=(0.0, 1e-2, 1e-4))
    assert e.value.status == "InvalidArgument"


def test_adjoint_surface_matches_bump_surface():
    """method="adjoint": one portfolio adjoint launch over the cells. On a
    European call (no barrier to smooth) the pathwise delta and vega agree
    with CRN central differences of relative size 1e-6 (the kink of the payoff
    contributes O(h)), and the prices are each cell's plain price."""
    c = kx.european_call("X", 100.0, 1.0)
    spots, vols = [90.0, 100.0, 110.0], [0.15, 0.3]
    a = kx.greek_surface(c, "X", spots, vols, n_paths=200_000, seed=4, steps_per_year=1, rate=R, method="adjoint",
                         precision="fp64")
    b = kx.greek_surface(c, "X", spots, vols, n_paths=200_000, seed=4, steps_per_year=1, rate=R,
                         bumps=(1e-6, 1e-6, 1e-6), relative=True, precision="fp64")
    assert all(math.isnan(x) for x in a.gamma.ravel())
    for i, sp in enumerate(spots):
        for j, v in enumerate(vols):
            p = c.price(kx.GBM(s0=sp, sigma=v, r=R, asset="X"), n_paths=200_000, seed=4, steps_per_year=1,
                        precision="fp64")
            assert abs(a.price[i, j] - p.price) <= 1e-12 * p.price
            for q in ("delta", "vega", "rho"):
                assert abs(getattr(a, q)[i, j] - getattr(b, q)[i, j]) <= 2e-5 * max(1.0, abs(getattr(b, q)[i, j])), \
                    (sp, v, q, getattr(a, q)[i, j], getattr(b, q)[i, j])
    with pytest.raises(kx.KontractError) as e:
        kx.greek_surface(c, "X", [], [0.2], method="adjoint")
    assert e.value.status == "InconsistentPath"

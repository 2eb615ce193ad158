"""Greek surfaces on the CPU: the oracle's greek_surface against the
reference's own checks (tests/surface.rs): dimensions, delta within 2 % and
vega within 3 % of Black-Scholes on a 3 x 3 grid, delta increasing with the
spot, an empty grid rejected; and the host-side exports of GreekSurface
(surface.rs:38-97) on known matrices."""
import math

import pytest

import kontracts_gb300 as kx
from oracle import OracleError

K, R, T = 100.0, 0.05, 1.0


def _call():
    # european_call of tests/surface.rs:38-43
    return kx.european_call("AAPL", K, T)


def _surface(orc, spots, vols, bumps=(1e-2, 1e-2, 1e-4), n_paths=200_000):
    # cfg() of tests/surface.rs:45-53
    cells = orc.greek_surface(_call().to_json(), "AAPL", spots, vols, n_paths=n_paths, seed=2024,
                              steps_per_year=1, rate=R, bumps=bumps)

    class _G:
        def __init__(self, d):
            self.__dict__.update(d)
    return kx.GreekSurface(spots, vols, [_G(d) for d in cells])


def _bs_delta_vega(s, k, r, sigma, t):
    d1 = (math.log(s / k) + (r + 0.5 * sigma * sigma) * t) / (sigma * math.sqrt(t))
    nd1 = 0.5 * (1.0 + math.erf(d1 / math.sqrt(2.0)))
    pdf = math.exp(-0.5 * d1 * d1) / math.sqrt(2.0 * math.pi)
    return nd1, s * pdf * math.sqrt(t)


def test_surface_dimensions_are_consistent(orc):
    s = _surface(orc, [90.0, 100.0, 110.0], [0.15, 0.20, 0.25], bumps=(1.0, 1e-2, 1e-4), n_paths=20_000)
    for q in ("price", "delta", "gamma", "vega"):
        assert getattr(s, q).shape == (3, 3)


def test_delta_and_vega_surfaces_match_black_scholes(orc):
    spots, vols = [90.0, 100.0, 110.0], [0.15, 0.20, 0.25]
    s = _surface(orc, spots, vols, bumps=(1.0, 1e-2, 1e-4))
    for i, sp in enumerate(spots):
        for j, v in enumerate(vols):
            d_bs, v_bs = _bs_delta_vega(sp, K, R, v, T)
            assert abs(s.delta[i, j] - d_bs) / d_bs < 0.02, (sp, v)
            assert abs(s.vega[i, j] - v_bs) / v_bs < 0.03, (sp, v)


def test_delta_increases_with_spot(orc):
    s = _surface(orc, [80.0, 100.0, 120.0], [0.20])
    assert s.delta[0, 0] < s.delta[1, 0] < s.delta[2, 0]


def test_cells_are_greeks_at_the_cell(orc):
    """Each cell is greeks_gbm at (spots[i], vols[j]) (surface.rs:120-124)."""
    spots, vols = [95.0, 105.0], [0.18, 0.22]
    cells = orc.greek_surface(_call().to_json(), "AAPL", spots, vols, n_paths=5_000, seed=7, steps_per_year=4,
                              rate=R)
    for i, sp in enumerate(spots):
        for j, v in enumerate(vols):
            g = orc.greeks(_call().to_json(), kx.GBM(s0=sp, sigma=v, r=R, asset="AAPL"), n_paths=5_000, seed=7,
                           steps_per_year=4)
            assert cells[i * len(vols) + j] == g


def test_empty_grid_is_rejected(orc):
    for spots, vols in (([], [0.2]), ([100.0], [])):
        with pytest.raises(OracleError) as e:
            orc.greek_surface(_call().to_json(), "AAPL", spots, vols, n_paths=100, steps_per_year=1, rate=R)
        assert e.value.code == 4  # InconsistentPath


def test_csv_and_pgm_exports_are_well_formed(orc):
    """tests/surface.rs:133-153."""
    s = _surface(orc, [95.0, 105.0], [0.18, 0.22], n_paths=20_000)
    csv = s.to_csv(s.delta)
    assert csv.startswith("spot\\vol,0.18,0.22")
    assert len(csv.splitlines()) == 3
    assert s.to_pgm(s.delta).startswith("P2\n2 2\n255")


class _Cell:
    def __init__(self, x):
        for q in kx.GreekSurface.QUANTITIES:
            setattr(self, q, x)


def test_csv_formats_like_rust_display():
    """`{}` of an f64: integral values without a fraction, no exponent."""
    s = kx.GreekSurface([95.0, 1e-7], [0.1, 1e21], [_Cell(x) for x in (0.30000000000000004, -0.0, 2.5, math.nan)])
    assert s.to_csv(s.price) == "spot\\vol,0.1,1000000000000000000000\n" \
                                "95,0.30000000000000004,-0\n0.0000001,2.5,NaN\n"


def test_pgm_normalises_min_to_max():
    """Values map to round((x - lo) / (hi - lo) * 255), half away from zero;
    a flat matrix maps to 0."""
    s = kx.GreekSurface([1.0, 2.0], [1.0, 2.0, 3.0], [_Cell(x) for x in (0.0, 0.5 / 255, 1.0, 2.0, 3.0, 4.0)])
    assert s.to_pgm(s.price) == "P2\n3 2\n255\n0 0 64 \n128 191 255 \n"
    flat = kx.GreekSurface([1.0], [1.0, 2.0], [_Cell(7.0), _Cell(7.0)])
    assert flat.to_pgm(flat.price) == "P2\n2 1\n255\n0 0 \n"

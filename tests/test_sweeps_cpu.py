"""Host logic of the experiment sweeps and the serving request stream (no GPU):
the sweep points follow the reference's drivers (src/main.py:150-207) and
post-processing starts (src/visualizations_utils.py:135-260); a seeded request
stream has the same requests at every offered rate."""
import numpy as np
import pytest

from lattice_boltzmann_parallel_solver_gb300 import serving, sweeps


def test_reynolds_points():
    pts = sweeps.sweep_points("reynolds")
    assert [p["label"] for p in pts] == [40, 70, 100, 140, 170, 200]
    for p in pts:
        assert (p["lx"], p["ly"]) == (420, 180)
        re_ = p["label"]
        if re_ > 130:
            assert p["nu"] == 0.03 and p["u"] == re_ * 0.03 / 40
        else:
            assert p["u"] == 0.1 and p["nu"] == 40 * 0.1 / re_
        # Re = plate u / nu (experiments.py:708)
        assert 40 * p["u"] / p["nu"] == pytest.approx(re_)
    assert [p["start"] for p in pts] == [150000, 125000, 70000, 70000, 70000, 70000]


def test_length_and_blockage_points():
    pts = sweeps.sweep_points("nx")
    assert [p["lx"] for p in pts] == [260, 300, 350, 420, 500, 750, 1000, 1250]
    assert all(p["ly"] == 180 and p["nu"] == 0.04 and p["u"] == 0.1 for p in pts)
    assert [p["start"] for p in pts] == [125000, 90000, 90000, 75000, 75000, 75000, 75000, 75000]
    pts = sweeps.sweep_points("blockage")
    assert [p["ly"] for p in pts] == [60, 100, 140, 180, 260]
    assert [p["label"] for p in pts] == [40 / ly for ly in (60, 100, 140, 180, 260)]
    with pytest.raises(ValueError):
        sweeps.sweep_points("width")


def test_request_stream_is_the_same_at_every_rate():
    a = serving.request_stream(60, rate=5.0, seed=7)
    b = serving.request_stream(60, rate=20.0, seed=7)
    assert [r[2:] for r in a] == [r[2:] for r in b]
    ta, tb = np.array([r[1] for r in a]), np.array([r[1] for r in b])
    assert np.allclose(ta, 4.0 * tb, rtol=1e-12) and np.all(np.diff(ta) > 0)
    assert {r[2] for r in a} == {"couette", "poiseuille", "von_karman"}
    for rid, t, kind, steps, nx, ny, params in a:
        assert 1000 <= steps <= 50000
        if kind == "couette":
            assert nx == ny and 32 <= ny <= 512 and 0.01 <= params["u_w"] <= 0.1
        elif kind == "poiseuille":
            assert 64 <= nx <= 2048 and 16 <= ny <= 512 and 1e-4 <= params["drho"] <= 1e-2
        else:
            assert (nx, ny) == (420, 180)


def test_next_admissions_respect_slots_and_budget():
    """The requests the serving loop prepares while the GPU runs a tick: the
    head of the queue that fits the free slots and the HBM budget, plus two."""
    from types import SimpleNamespace
    reqs = [SimpleNamespace(rid=k, size=100 * (k + 1)) for k in range(10)]
    eng = SimpleNamespace(used=0, max_slots=4, live=[], hbm_budget=10 ** 9,
                          state_bytes=lambda r: r.size)
    take = serving.ServingEngine._next_admissions
    assert [r.rid for r in take(eng, reqs)] == [0, 1, 2, 3, 4, 5]      # 4 slots + 2
    eng.live = [None] * 4
    assert [r.rid for r in take(eng, reqs)] == [0, 1]                  # no slot free
    eng.live, eng.hbm_budget = [], 350
    assert [r.rid for r in take(eng, reqs)] == [0, 1, 2, 3]            # 100 + 200 fit, then 2 more
    assert take(eng, []) == []

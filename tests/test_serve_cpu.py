"""Host-side logic of the server and the batch generator (no GPU)."""
import numpy as np
import pytest

from dustyshock3d_gb300 import ic
from dustyshock3d_gb300.serve import Server, grid_sizes, memory_estimate, poisson_requests
from oracle.oracle import OracleState


def test_grid_sizes_match_oracle():
    for P, sp in [ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, x_range=(-0.25, 0.25)),
                  ic.dusty_sod_tube(dx_left=1 / 200, Ly=0.1)]:
        info = OracleState(P, sp).grid_info()
        nc, ni = grid_sizes(P)
        assert nc == info[3] and ni == info[7]


def test_memory_estimate_scales_with_particles():
    P1, s1 = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, x_range=(-0.25, 0.25))
    P2, s2 = ic.dusty_sod_tube(dx_left=1 / 128, Ly=0.25, x_range=(-0.25, 0.25))
    assert memory_estimate(P2, s2) > 4 * memory_estimate(P1, s1)


def test_poisson_arrivals_seeded():
    mk = lambda rng: ic.dusty_sod_tube(dx_left=1 / 32, Ly=0.25, x_range=(-0.25, 0.25))  # noqa: E731
    a = poisson_requests(5.0, 6, 7, mk)
    b = poisson_requests(5.0, 6, 7, mk)
    assert [r.arrival for r in a] == [r.arrival for r in b]
    assert all(0.05 <= r.t_end <= 0.2 for r in a)
    assert np.all(np.diff([r.arrival for r in a]) > 0)


def test_batch_distributions():
    rng = np.random.default_rng(1)
    d = [ic.draw_tube_params(rng) for _ in range(2000)]
    n = np.array([x["N_gas"] for x in d])
    assert n.min() >= 2e4 and n.max() <= 1e6
    assert 4 <= min(x["rho_ratio"] for x in d) and max(x["rho_ratio"] for x in d) <= 16
    assert 5 <= min(x["p_ratio"] for x in d) and max(x["p_ratio"] for x in d) <= 20
    e = np.log10([x["eps"] for x in d])
    assert -2 <= e.min() and e.max() <= 1 and abs(np.median(e) + 0.5) < 0.1


def test_fp32_estimate_counts_force_lists():
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, x_range=(-0.25, 0.25))
    P.precision = "fp32"
    on = memory_estimate(P, sp)
    P.force_list = -1
    off = memory_estimate(P, sp)
    assert on - off >= sp[0].n * 4 * 256


def test_request_larger_than_budget_is_refused():
    """A request that cannot fit even an empty server raises instead of
    waiting for room that never comes (no GPU work happens before)."""
    mk = lambda rng: ic.dusty_sod_tube(dx_left=1 / 32, Ly=0.25, x_range=(-0.25, 0.25))  # noqa: E731
    reqs = poisson_requests(1e6, 2, 3, mk)
    server = Server(budget_bytes=0.5 * Server(precision="fp32").estimate(reqs[0]), precision="fp32")
    with pytest.raises(ValueError, match="budget"):
        server.run(reqs)


def test_device_generated_request_counts_and_estimate():
    from dustyshock3d_gb300 import ic
    from dustyshock3d_gb300.serve import Request, device_uneven_tube
    kw = dict(N_gas=3e4, rho_ratio=8.0, p_ratio=10.0, eps=1.0, t_s=1e-3)
    P, sp = ic.uneven_tube(**kw)
    spec = ic.DeviceIC.uneven(**kw)
    r_host = Request(0, 0.0, P, sp, 0.1)
    r_dev = Request(1, 0.0, spec.plan()[0], None, 0.1, ic=spec)
    assert r_dev.counts == r_host.counts and r_dev.particles == r_host.particles
    srv = Server(precision="fp32")
    assert srv.estimate(r_dev) == srv.estimate(r_host)
    # the seeded stream draws the same tubes either way
    import numpy as np
    a = device_uneven_tube(np.random.default_rng(5))
    b_params, b_species = ic.uneven_tube(**ic.draw_tube_params(np.random.default_rng(5)))
    assert a[1].plan()[1] == [s.n for s in b_species]

"""Continuous batching: requests that join and leave a running batch get the
same result as when solved alone (bit for bit: a tube's arithmetic does not
depend on the other tubes of its batch)."""
import numpy as np
import pytest

from dustyshock3d_gb300 import ic
from dustyshock3d_gb300.serve import Request, Server, one_at_a_time, run_alone

pytestmark = pytest.mark.gpu


def _requests():
    shapes = [dict(eps=1.0, t_s=1e-3), dict(eps=0.1, t_s=1e-2, rho_R=0.25, p_R=0.2),
              dict(eps=3.0, t_s=3e-4), dict(eps=0.5, t_s=5e-2, rho_R=0.1, p_R=0.125)]
    out = []
    for i, kw in enumerate(shapes):
        P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, x_range=(-0.25, 0.25), **kw)
        out.append(Request(i, 0.05 * i, P, sp, t_end=0.012 + 0.006 * i))
    return out


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_mix_equals_alone(precision):
    reqs = _requests()
    server = Server(budget_bytes=150e9, epoch_steps=2, precision=precision)
    results = server.run(reqs)
    assert [r.rid for r in results] == [0, 1, 2, 3]
    assert server.rebuilds >= 2, "requests should have joined a running batch"
    for req, res in zip(reqs, results):
        alone = run_alone(req, precision)
        for s in range(2):
            for f in ("x", "y", "z", "vx", "vy", "vz", "rho"):
                a, b = getattr(res.species[s], f), getattr(alone[s], f)
                assert np.array_equal(a, b), f"request {req.rid} species {s} {f}"
        assert res.time_to_solution >= 0


def test_budget_admits_one_at_a_time():
    reqs = _requests()[:3]
    one = max(Server(precision="fp32").estimate(r) for r in reqs)
    server = Server(budget_bytes=1.2 * one, epoch_steps=4, precision="fp32")
    results = server.run(reqs)
    assert len(results) == 3
    # never two tubes at once: each admitted after the previous finished
    order = sorted(results, key=lambda r: r.admitted)
    for a, b in zip(order, order[1:]):
        assert b.admitted >= a.finished - 1e-9
    for req, res in zip(reqs, results):
        alone = run_alone(req, "fp32")
        assert np.array_equal(res.species[0].rho, alone[0].rho)


def test_device_generated_requests_equal_uploaded_requests():
    """Requests whose particles the server generates on the device at admission
    (ds_init_tube) finish with the same particles as the same tubes made on the
    host and uploaded."""
    shapes = [dict(N_gas=2.5e4, rho_ratio=8.0, p_ratio=10.0, eps=1.0, t_s=1e-3),
              dict(N_gas=4.0e4, rho_ratio=5.0, p_ratio=7.0, eps=0.2, t_s=2e-2),
              dict(N_gas=1.5e4, rho_ratio=12.0, p_ratio=15.0, eps=3.0, t_s=4e-4)]
    host, dev = [], []
    for i, kw in enumerate(shapes):
        t_end = 0.01 + 0.005 * i
        P, sp = ic.uneven_tube(**kw)
        host.append(Request(i, 0.05 * i, P, sp, t_end=t_end))
        spec = ic.DeviceIC.uneven(**kw)
        dev.append(Request(i, 0.05 * i, spec.plan()[0], None, t_end=t_end, ic=spec))
    a = Server(budget_bytes=150e9, epoch_steps=2, precision="fp32").run(host)
    b = Server(budget_bytes=150e9, epoch_steps=2, precision="fp32").run(dev)
    for ra, rb in zip(a, b):
        assert ra.steps == rb.steps and ra.particles == rb.particles
        for s in range(2):
            for f in ("x", "y", "z", "vx", "vy", "vz", "rho", "ind"):
                assert np.array_equal(getattr(ra.species[s], f), getattr(rb.species[s], f)), (ra.rid, s, f)


def test_one_at_a_time_comparator_equals_the_served_results():
    """The measured one-at-a-time comparator (serve.one_at_a_time) solves each
    request alone, in arrival order: the same particles as the served mix, and
    no request starts before the previous one finished."""
    reqs = _requests()[:3]
    served = Server(budget_bytes=150e9, epoch_steps=2, precision="fp32").run(reqs)
    seq = one_at_a_time(reqs, "fp32", group=2)
    for a, b in zip(served, seq):
        assert a.rid == b.rid and a.steps == b.steps
        for s in range(2):
            assert np.array_equal(a.species[s].vx, b.species[s].vx) and np.array_equal(a.species[s].x, b.species[s].x)
    order = sorted(seq, key=lambda r: r.arrival)
    for x, y in zip(order, order[1:]):
        assert y.admitted >= x.finished - 1e-9 and y.admitted >= y.arrival - 1e-9

"""Parameter derivatives (tis_param_grad) and the reverse pass through fixed-noise
trajectories (tis_traj_grad) against central finite differences of the engine's
own FP64 path, on the 76-nt test system.

Tolerance: 1e-4 relative to the finite difference, plus the difference's own
rounding floor (the FP64 force sums are atomics in arbitrary order, so a result
repeats only to ~1e-13 relative; that noise divided by the step is the floor)."""
import numpy as np
import pytest

from systems import golden_inputs, load
from tis_autograd import make_trajectory_function, params_of, run_final_state, with_params
from tis_gb300 import N_PARAMS, PARAM_NAMES, PREC_FP64, PREC_MIXED, STATE_NAMES, TERM_BONDED, TERM_HB, TERM_LR, \
    TERM_SR, TERM_STACK, Engine

ALL = TERM_SR | TERM_LR | TERM_BONDED | TERM_STACK | TERM_HB
U_TERMS = ["E_lj", "E_coul_sr", "E_coul_lr", "E_bond", "E_angle", "E_excl", "E2_STACK", "E3_STACK", "E2_HB", "E3_HB"]


@pytest.fixture(scope="module")
def small():
    return load(golden_inputs(), "small")


@pytest.fixture(scope="module")
def thermal(small):
    """A thermalized state of the small system: 300 FP64 steps from its set-up."""
    e = Engine([small], precision=PREC_FP64)
    e.populate_lists()
    e.step(300)
    e.sync()
    st = e.get_states()
    e.close()
    return st


def potential(system, theta, state, prec=PREC_FP64):
    """Total potential energy at `state` with parameters theta (a fresh engine: the
    H-bond term's Monte Carlo draws from the start of the replica's stream)."""
    e = Engine([with_params(system, theta)], precision=prec)
    e.set_states(state)
    e.populate_lists()
    _, en = e.forces(0, ALL)
    e.close()
    return sum(en[k] for k in U_TERMS), sum(abs(en[k]) for k in U_TERMS)


def param_grad(system, theta, state, prec=PREC_FP64):
    e = Engine([with_params(system, theta)], precision=prec)
    e.set_states(state)
    g = e.param_grad()[0]
    e.close()
    return g


@pytest.mark.gpu
def test_param_grad_matches_finite_differences(small, thermal):
    """dU/dtheta of all 16 parameters at a thermal frame against central differences
    (h = 1e-4 relative) of the engine's total FP64 energy."""
    th0 = params_of(small)
    g = param_grad(small, th0, thermal)
    u0, uabs = potential(small, th0, thermal)
    u1, _ = potential(small, th0, thermal)
    noise = max(abs(u1 - u0), 1e-14 * uabs)
    rows = []
    for j in range(N_PARAMS):
        if th0[j] == 0.0:  # the Debye length of an unscreened system: no derivative
            assert g[j] == 0.0, PARAM_NAMES[j]
            continue
        hj = 1e-4 * abs(th0[j])
        tp, tm = th0.copy(), th0.copy()
        tp[j] += hj
        tm[j] -= hj
        fd = (potential(small, tp, thermal)[0] - potential(small, tm, thermal)[0]) / (2 * hj)
        tol = 1e-4 * abs(fd) + 10 * noise / hj
        rows.append(f"{PARAM_NAMES[j]} adj {g[j]:+.9e} fd {fd:+.9e}")
        assert abs(g[j] - fd) <= tol, rows[-1]
    print("\n".join(rows))
    assert np.count_nonzero(g) >= 12  # every class of term is present in this system


def oracle_potential(system, theta, state):
    """The FP64 oracle's total potential energy at `state` with parameters theta."""
    from oracle_bridge import Oracle
    o = Oracle(with_params(system, theta).to_dict(), seed=int(system["seed"][0]))
    o.set_state(state)
    o.populate_lists()
    t = o.terms()
    return sum(t[k] for k in U_TERMS)


@pytest.mark.gpu
def test_param_grad_matches_oracle_finite_differences(small, thermal):
    """The reference gradient: central differences (h = 1e-4 relative) of the CPU
    oracle's FP64 total energy, the oracle being the reference's algorithm pinned
    to the reference's own outputs."""
    th0 = params_of(small)
    g = param_grad(small, th0, thermal)
    u0 = oracle_potential(small, th0, thermal)
    rows = []
    for j in range(N_PARAMS):
        if th0[j] == 0.0:  # the Debye length of an unscreened system: no derivative
            assert g[j] == 0.0, PARAM_NAMES[j]
            continue
        hj = 1e-4 * abs(th0[j])
        tp, tm = th0.copy(), th0.copy()
        tp[j] += hj
        tm[j] -= hj
        fd = (oracle_potential(small, tp, thermal) - oracle_potential(small, tm, thermal)) / (2 * hj)
        tol = 1e-4 * abs(fd) + 1e-14 * abs(u0) / hj
        rows.append(f"{PARAM_NAMES[j]:7s} adj {g[j]:+.9e} oracle fd {fd:+.9e}")
        assert abs(g[j] - fd) <= tol, rows[-1]
    print("\n".join(rows))


@pytest.mark.gpu
def test_param_grad_mixed_equals_fp64(small, thermal):
    """The derivatives are FP64 in both engine precisions; only the H-bond Monte
    Carlo, decided by each precision's energies, could differ (it does not here)."""
    th0 = params_of(small)
    a = param_grad(small, th0, thermal, PREC_FP64)
    b = param_grad(small, th0, thermal, PREC_MIXED)
    np.testing.assert_allclose(b, a, rtol=1e-9, atol=1e-9 * np.abs(a).max())


def _loss_seed(n, rng):
    return {k: rng.standard_normal(n) for k in ("x", "y", "z", "vx", "vy", "vz")}


def _loss(state, seed):
    return sum(float(np.dot(state[k], w)) for k, w in seed.items())


@pytest.mark.gpu
@pytest.mark.parametrize("steps,every", [(40, 10), (23, 7)])
def test_traj_grad_matches_finite_differences(small, thermal, steps, every):
    """dL/dtheta and dL/dx0 through `steps` fixed-noise FP64 steps (list rebuilds
    and LR refreshes included) against central differences of L = w . (x_T, v_T).
    Steps: 1e-3 relative for the parameters that enter as factors (the difference
    is then exact up to rounding), 1e-4 for the ion radii (whose truncation error,
    h^2, is 1e-4 relative at h = 1e-3); floor: FP64 rounding of L (1e-14 |L|)
    divided by the step."""
    th0 = params_of(small)
    n = thermal["x"].size
    rng = np.random.default_rng(11)
    seed = _loss_seed(n, rng)
    e = Engine([with_params(small, th0)], precision=PREC_FP64)
    e.set_states(thermal)
    dth, d0 = e.traj_grad(steps, every, seed, want_state=True)
    fin = e.get_states()
    e.close()
    ref = run_final_state(small, th0, thermal, steps, precision=PREC_FP64)
    for k in STATE_NAMES:  # tis_traj_grad leaves the forward pass's final state
        np.testing.assert_allclose(fin[k], ref[k], rtol=0, atol=1e-9)
    L = [_loss(ref, seed)] + [_loss(run_final_state(small, th0, thermal, steps, precision=PREC_FP64), seed)
                              for _ in range(3)]
    noise = max(max(L) - min(L), 1e-14 * abs(L[0]))
    rows = [f"L {L[0]:.6e}, spread over 4 runs {max(L) - min(L):.2e}"]
    worst = 0.0
    for j in range(N_PARAMS):
        if th0[j] == 0.0:  # the Debye length of an unscreened system: no derivative
            assert dth[0, j] == 0.0, PARAM_NAMES[j]
            continue
        hj = (1e-4 if PARAM_NAMES[j].startswith("R_") else 1e-3) * abs(th0[j])
        tp, tm = th0.copy(), th0.copy()
        tp[j] += hj
        tm[j] -= hj
        fd = (_loss(run_final_state(small, tp, thermal, steps, precision=PREC_FP64), seed) -
              _loss(run_final_state(small, tm, thermal, steps, precision=PREC_FP64), seed)) / (2 * hj)
        floor = noise / hj
        tol = 1e-4 * abs(fd) + floor
        rows.append(f"{PARAM_NAMES[j]:7s} adj {dth[0, j]:+.9e} fd {fd:+.9e} diff {abs(dth[0, j] - fd):.1e} "
                    f"floor {floor:.1e}")
        if floor < 1e-5 * abs(fd):
            worst = max(worst, abs(dth[0, j] - fd) / abs(fd))
        assert abs(dth[0, j] - fd) <= tol, rows[-1]
    # a random direction of the initial positions
    delta = {k: rng.standard_normal(n) for k in ("x", "y", "z")}
    h = 1e-6
    sp = {k: thermal[k] + h * delta[k] if k in delta else thermal[k] for k in STATE_NAMES}
    sm = {k: thermal[k] - h * delta[k] if k in delta else thermal[k] for k in STATE_NAMES}
    fd = (_loss(run_final_state(small, th0, sp, steps, precision=PREC_FP64), seed) -
          _loss(run_final_state(small, th0, sm, steps, precision=PREC_FP64), seed)) / (2 * h)
    ad = sum(float(np.dot(d0[k], delta[k])) for k in delta)
    rows.append(f"x0 direction adj {ad:+.9e} fd {fd:+.9e}")
    rows.append(f"largest relative difference where the floor is below 1e-5 of it: {worst:.2e}")
    print("\n".join(rows))
    assert abs(ad - fd) <= 1e-4 * abs(fd) + noise / h, rows[-2]


def oracle_final_state(system, theta, state, steps):
    from oracle_bridge import Oracle
    o = Oracle(with_params(system, theta).to_dict(), seed=int(system["seed"][0]))
    o.set_state(state)
    o.populate_lists()
    o.step(steps)
    return o.get_state()


@pytest.mark.gpu
def test_traj_grad_matches_oracle_finite_differences(small, thermal):
    """The reference gradient through 40 fixed-noise steps: central differences of
    L = w . (x_T, v_T) over the CPU oracle's own trajectories (the reference's
    algorithm and rand() stream), against tis_traj_grad on the FP64 engine."""
    th0 = params_of(small)
    seed = _loss_seed(thermal["x"].size, np.random.default_rng(11))
    e = Engine([with_params(small, th0)], precision=PREC_FP64)
    e.set_states(thermal)
    dth = e.traj_grad(40, 10, seed)[0]
    e.close()
    L0 = _loss(oracle_final_state(small, th0, thermal, 40), seed)
    rows = []
    for j in range(N_PARAMS):
        if th0[j] == 0.0:  # the Debye length of an unscreened system: no derivative
            assert dth[j] == 0.0, PARAM_NAMES[j]
            continue
        hj = (1e-4 if PARAM_NAMES[j].startswith("R_") else 1e-3) * abs(th0[j])
        tp, tm = th0.copy(), th0.copy()
        tp[j] += hj
        tm[j] -= hj
        fd = (_loss(oracle_final_state(small, tp, thermal, 40), seed) -
              _loss(oracle_final_state(small, tm, thermal, 40), seed)) / (2 * hj)
        tol = 1e-4 * abs(fd) + 1e-14 * abs(L0) / hj
        rows.append(f"{PARAM_NAMES[j]:7s} adj {dth[j]:+.9e} oracle fd {fd:+.9e}")
        assert abs(dth[j] - fd) <= tol, rows[-1]
    print("\n".join(rows))


@pytest.mark.gpu
def test_traj_grad_batch_equals_single(synth_dir):
    """Three replicas (different seeds and ion counts) in two replica groups give
    each replica the gradient it has alone; the packed dL/dx0 lands at each
    replica's offset."""
    systems = [load(synth_dir["small"], "small", seed=s, n_mg=m) for s, m in ((3, 10), (4, 20), (5, 0))]
    ns = []
    states = []
    for s in systems:
        e = Engine([s], precision=PREC_FP64)
        e.populate_lists()
        e.step(100)
        e.sync()
        states.append(e.get_states())
        ns.append(states[-1]["x"].size)
        e.close()
    rng = np.random.default_rng(2)
    seeds = [_loss_seed(n, rng) for n in ns]
    single = []
    for s, st, sd in zip(systems, states, seeds):
        e = Engine([s], precision=PREC_FP64)
        e.set_states(st)
        single.append(e.traj_grad(15, 4, sd, want_state=True))
        e.close()
    e = Engine(systems, precision=PREC_FP64, groups=2)
    e.set_states({k: np.concatenate([st[k] for st in states]) for k in STATE_NAMES})
    seed = {k: np.concatenate([sd[k] for sd in seeds]) for k in seeds[0]}
    dth, d0 = e.traj_grad(15, 4, seed, want_state=True)
    e.close()
    off = 0
    for r, (g1, s1) in enumerate(single):
        np.testing.assert_allclose(dth[r], g1[0], rtol=1e-8, atol=1e-10 * np.abs(g1[0]).max())
        for k in STATE_NAMES:
            np.testing.assert_allclose(d0[k][off:off + ns[r]], s1[k], rtol=1e-8,
                                       atol=1e-10 * (np.abs(s1[k]).max() + 1e-300))
        off += ns[r]


@pytest.mark.gpu
def test_traj_grad_mixed_forward_close_to_fp64(small, thermal):
    """The mixed-precision forward (FP32 pair math, fixed-point sums) under the FP64
    adjoint: the gradient differs from the FP64 path's by the trajectory's own
    precision difference."""
    th0 = params_of(small)
    seed = _loss_seed(thermal["x"].size, np.random.default_rng(3))
    out = {}
    for name, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
        e = Engine([with_params(small, th0)], precision=prec)
        e.set_states(thermal)
        out[name] = e.traj_grad(40, 10, seed)[0]
        e.close()
    rel = np.abs(out["mixed"] - out["fp64"]) / np.maximum(np.abs(out["fp64"]), 1e-12)
    print("mixed vs fp64 relative difference per parameter:", np.array2string(rel, precision=1))
    big = np.abs(out["fp64"]) > 1e-3 * np.abs(out["fp64"]).max()
    assert rel[big].max() < 1e-3


@pytest.mark.gpu
def test_autograd_function_backward(small, thermal):
    """The torch.autograd.Function of the validation harness: backward through
    tis_traj_grad equals the finite difference of its forward."""
    torch = pytest.importorskip("torch")
    steps, every = 20, 5
    fn, template = make_trajectory_function(small, steps, every, precision=PREC_FP64)
    template.update(thermal)
    theta = torch.tensor(params_of(small), dtype=torch.float64, requires_grad=True)
    x0 = torch.tensor(np.stack([thermal["x"], thermal["y"], thermal["z"]]), dtype=torch.float64, requires_grad=True)
    w = torch.tensor(np.random.default_rng(5).standard_normal(x0.shape), dtype=torch.float64)
    loss = (fn.apply(theta, x0) * w).sum()
    loss.backward()
    j = 14  # lB
    hj = 1e-3 * float(theta.detach()[j])
    with torch.no_grad():
        tp, tm = theta.detach().clone(), theta.detach().clone()
        tp[j] += hj
        tm[j] -= hj
        fd = ((fn.apply(tp, x0.detach()) * w).sum() - (fn.apply(tm, x0.detach()) * w).sum()) / (2 * hj)
    assert float(theta.grad[j]) == pytest.approx(float(fd), rel=1e-4)
    assert x0.grad.shape == x0.shape and torch.isfinite(x0.grad).all()

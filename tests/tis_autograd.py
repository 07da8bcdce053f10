"""Validation harness for the adjoint: the force-field parameter vector of a
system (tis_gb300.PARAM_NAMES order), systems rebuilt at other parameter values,
and a torch.autograd.Function over a fixed-noise trajectory whose backward is
the engine's tis_traj_grad.  Test infrastructure only."""
import numpy as np

from tis_gb300 import N_PARAMS, STATE_NAMES, Engine, System

# MAXIKEY types (0-based rows of elj / rlj) of each LJ epsilon parameter (6..11)
EPS_TYPES = [[0], [1], [2, 3, 4, 5], [6], [7], [8]]


def debye_of(system):
    """The system's Debye length (0: unscreened, the reference's Coulomb)."""
    d = system.to_dict()
    return float(np.asarray(d["debye"]).ravel()[0]) if "debye" in d else 0.0


def params_of(system):
    """theta of a loaded system: ss_D (x4), st_D, hs_D, ELJ of P S B Mg Cl K, RLJ of Mg K, lB,
    Debye length."""
    ss, st, hs = (float(system[k][0]) for k in ("ss_D", "st_D", "hs_D"))
    elj, rlj = system["elj"], system["rlj"]
    eps = [float(elj[t[0]]) for t in EPS_TYPES]
    return np.array([ss] * 4 + [st, hs] + eps + [float(rlj[6]), float(rlj[8]), float(system["lB"][0]),
                                                 debye_of(system)])


def screened(system, debye):
    """A copy of `system` with the Debye length of its Coulomb term set (0: unscreened)."""
    arrays = system.to_dict()
    arrays["debye"] = np.array([float(debye)])
    return System.from_arrays(arrays)


def with_params(system, theta):
    """A copy of `system` whose parameter-dependent arrays are those of theta (the
    linear dependences of st2_E, st3_E and hb_E, E:4344, E:4397-4427, E:3881)."""
    base = params_of(system)
    arrays = system.to_dict()
    st2 = arrays["st2_E"].copy()
    for c in range(4):
        sel = arrays["st2_cls"] == c
        st2[sel] += (theta[c] - base[c]) * arrays["st2_dss"][sel]
    arrays["st2_E"] = st2
    arrays["st3_E"] = np.full_like(arrays["st3_E"], -theta[4])
    arrays["hb_E"] = arrays["hb_E"] + (theta[5] - base[5]) * arrays["hb_dhs"]
    elj = arrays["elj"].copy()
    for k, types in enumerate(EPS_TYPES):
        elj[types] = theta[6 + k]
    arrays["elj"] = elj
    rlj = arrays["rlj"].copy()
    rlj[6], rlj[8] = theta[12], theta[13]
    arrays["rlj"] = rlj
    arrays["lB"] = np.array([theta[14]])
    arrays["debye"] = np.array([theta[15]])
    arrays["ss_D"] = np.array([theta[0]])
    arrays["st_D"] = np.array([theta[4]])
    arrays["hs_D"] = np.array([theta[5]])
    return System.from_arrays(arrays)


def run_final_state(system, theta, state0, steps, **engine_kw):
    """State (packed dict) after `steps` steps from state0, the run starting with a list build."""
    e = Engine([with_params(system, theta)], **engine_kw)
    e.set_states(state0)
    e.populate_lists()
    e.step(steps)
    e.sync()
    out = e.get_states()
    e.close()
    return out


def make_trajectory_function(system, steps, checkpoint_every, **engine_kw):
    """torch.autograd.Function: (theta, x0 positions) -> final positions, through
    `steps` fixed-noise Langevin steps; backward through tis_traj_grad."""
    import torch

    class Trajectory(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, x0):
            th = theta.detach().cpu().numpy().astype(np.float64)
            st = {k: v for k, v in state_template.items()}
            xyz = x0.detach().cpu().numpy().astype(np.float64)
            st["x"], st["y"], st["z"] = xyz[0].copy(), xyz[1].copy(), xyz[2].copy()
            ctx.save_for_backward(theta, x0)
            fin = run_final_state(system, th, st, steps, **engine_kw)
            return torch.as_tensor(np.stack([fin["x"], fin["y"], fin["z"]]), dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad):
            theta, x0 = ctx.saved_tensors
            th = theta.detach().cpu().numpy().astype(np.float64)
            st = {k: v for k, v in state_template.items()}
            xyz = x0.detach().cpu().numpy().astype(np.float64)
            st["x"], st["y"], st["z"] = xyz[0].copy(), xyz[1].copy(), xyz[2].copy()
            g = grad.detach().cpu().numpy().astype(np.float64)
            e = Engine([with_params(system, th)], **engine_kw)
            e.set_states(st)
            dth, d0 = e.traj_grad(steps, checkpoint_every, {"x": g[0], "y": g[1], "z": g[2]}, want_state=True)
            e.close()
            dx0 = np.stack([d0["x"], d0["y"], d0["z"]])
            return torch.as_tensor(dth[0], dtype=theta.dtype), torch.as_tensor(dx0, dtype=x0.dtype)

    state_template = {}
    return Trajectory, state_template


assert N_PARAMS == 16 and len(STATE_NAMES) == 9

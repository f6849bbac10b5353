"""Speed misfit J = ½ Σ_h (|u| − u_obs)² over the ice cells (the adjoint workload's objective) and its
gradient with respect to the velocities, in numpy.  |u| is the depth-averaged speed on the h grid as
update_av_speed! forms it (update_velocities.jl:216-220): the masked u, v averaged to cell centres."""
import numpy as np


def speed(u, v, u_mask, v_mask, h_mask):
    um = np.where(u_mask, u, 0.0)
    vm = np.where(v_mask, v, 0.0)
    uc = np.where(h_mask, 0.5 * (um[:-1, :] + um[1:, :]), 0.0)
    vc = np.where(h_mask, 0.5 * (vm[:, :-1] + vm[:, 1:]), 0.0)
    return np.sqrt(uc * uc + vc * vc), uc, vc


def misfit(u, v, u_mask, v_mask, h_mask, s_obs):
    s, _, _ = speed(u, v, u_mask, v_mask, h_mask)
    r = np.where(h_mask, s - s_obs, 0.0)
    return 0.5 * float(np.sum(r * r))


def misfit_gradient(u, v, u_mask, v_mask, h_mask, s_obs):
    """(dJ/du, dJ/dv) in the reference shapes ((nx+1, ny), (nx, ny+1))."""
    s, uc, vc = speed(u, v, u_mask, v_mask, h_mask)
    r = np.where(h_mask, s - s_obs, 0.0)
    with np.errstate(invalid="ignore", divide="ignore"):
        fu = np.where(s > 0, 0.5 * r * uc / s, 0.0)
        fv = np.where(s > 0, 0.5 * r * vc / s, 0.0)
    gu = np.zeros_like(u)
    gv = np.zeros_like(v)
    gu[:-1, :] += fu
    gu[1:, :] += fu
    gv[:, :-1] += fv
    gv[:, 1:] += fv
    return np.where(u_mask, gu, 0.0), np.where(v_mask, gv, 0.0)

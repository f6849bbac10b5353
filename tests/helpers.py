"""Shared test helpers: move the oracle's model state into GPU-solver field dicts."""
import numpy as np

SOLVE_FIELDS = ("h", "s", "dsdh", "grounded_fraction", "weertman_c", "accumulation", "basal_melt", "gu_h", "gu_s",
                "gu_grounded_fraction", "gv_h", "gv_s", "gv_grounded_fraction", "glen_b", "u", "v", "eta", "beta",
                "quad_f2", "shelf_strain_rate", "av_speed", "bed_speed", "tau_bed", "eta_av", "quad_f1", "beta_eff",
                "gu_beta_eff", "gv_beta_eff")


def fields_from_oracle(om, g):
    f = {k: np.array(om.field(k), order="F") for k in SOLVE_FIELDS}
    f["gu_residual"] = np.array(om.field("gu_residual"), order="F")
    f["gv_residual"] = np.array(om.field("gv_residual"), order="F")
    f["wu_mask"] = np.array(om.mask("wu_mask"), order="F")
    f["wv_mask"] = np.array(om.mask("wv_mask"), order="F")
    wu = om.field("wu_correction_full")
    wv = om.field("wv_correction_full")
    # the compact coarse vectors list the masked points in column-major order (UWavelets.jl:46)
    f["wu_correction_coarse"] = np.array(np.asarray(wu).ravel(order="F")[f["wu_mask"].ravel(order="F") != 0])
    f["wv_correction_coarse"] = np.array(np.asarray(wv).ravel(order="F")[f["wv_mask"].ravel(order="F") != 0])
    return f


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


def uv_err(f, om):
    du = f["u"] - om.field("u")
    dv = f["v"] - om.field("v")
    num = np.sqrt(np.sum(du ** 2) + np.sum(dv ** 2))
    den = np.sqrt(np.sum(om.field("u") ** 2) + np.sum(om.field("v") ** 2))
    return num / den


def to_dev(f, torch):
    out = {}
    for k, a in f.items():
        flat = np.ascontiguousarray(np.asarray(a).ravel(order="F"))
        out[k] = torch.from_numpy(flat).cuda()
    return out


def from_dev(t, f):
    for k, a in f.items():
        host = t[k].cpu().numpy()
        if k in ("wu_correction_coarse", "wv_correction_coarse"):
            f[k] = host.copy()
        else:
            a[...] = host.reshape(a.shape, order="F")

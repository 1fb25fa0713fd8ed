"""Shared parity metrics: GPU results against the CPU oracle."""
import numpy as np

DEPTH_TOL = 1e-4        # scene units (the benchmark's depth tolerance)
MASK_AGREEMENT = 0.999  # fraction of samples with identical hit/miss


def compare_depth(t_gpu, m_gpu, t_ref, m_ref, quantile=0.999):
    mask_agree = float((m_gpu == m_ref).mean())
    both = (m_gpu == 1) & (m_ref == 1)
    if both.any():
        err = np.abs(t_gpu[both].astype(np.float64) - t_ref[both].astype(np.float64))
        q = float(np.quantile(err, quantile))
        mx = float(err.max())
        frac_ok = float((err <= DEPTH_TOL).mean())
    else:
        q = mx = 0.0
        frac_ok = 1.0
    return {"mask_agreement": mask_agree, "depth_err_q": q, "depth_err_max": mx, "depth_within_tol": frac_ok,
            "hits": int(both.sum())}


def assert_depth_parity(t_gpu, m_gpu, t_ref, m_ref, what=""):
    r = compare_depth(t_gpu, m_gpu, t_ref, m_ref)
    assert r["mask_agreement"] >= MASK_AGREEMENT, (what, r)
    assert r["depth_within_tol"] >= MASK_AGREEMENT, (what, r)
    return r


def radiance_rmse(a, b):
    """Root mean square of the radiance difference, in FP64."""
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)))

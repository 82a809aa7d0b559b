"""numpy restatement of the reference's pre-processing, REAL arithmetic with
member sums in order (src/letkf_state.F90:326-334, src/letkf_obs.F90:459-488).
Used by the CPU and GPU tests of the device-side preparation."""
import numpy as np

f32 = np.float32


def background_stats(members):
    """members [..., k] -> (perturbations, mean, spread)."""
    k = members.shape[-1]
    s = np.zeros(members.shape[:-1], f32)
    for m in range(k):
        s = (s + members[..., m]).astype(f32)
    mean = (s / f32(k)).astype(f32)
    pert = (members - mean[..., None]).astype(f32)
    dot = np.zeros(members.shape[:-1], f32)
    for m in range(k):
        dot = (dot + (pert[..., m] * pert[..., m]).astype(f32)).astype(f32)
    sprd = np.sqrt((dot / f32(k - 1)).astype(f32)).astype(f32)
    return pert, mean, sprd


def hx_stats(hx_members, qc=None):
    """hx_members [nobs, k] -> (perturbations, mean, keep mask), then the
    reference's order-preserving QC compaction is a boolean selection."""
    k = hx_members.shape[1]
    s = np.zeros(hx_members.shape[0], f32)
    for m in range(k):
        s = (s + hx_members[:, m]).astype(f32)
    mean = (s / f32(k)).astype(f32)
    pert = (hx_members - mean[:, None]).astype(f32)
    keep = np.ones(hx_members.shape[0], bool) if qc is None else ~(np.asarray(qc) > 0)
    return pert, mean, keep

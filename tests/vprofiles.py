"""Test helper: ViterbiFilter profiles cut to fewer nodes, for parity cases
at every row width of the GPU kernel."""
import numpy as np

from cudahmmsearch_gb300 import formats as F


def crop_vprofile(vp, M):
    """The first M nodes of a ViterbiFilter profile, restriped for Q8 =
    max(2, ceil(M/8)) (node k at vector (k-1) % Q8, element (k-1) // Q8).
    Nodes past M cost -32768 as the reference pads them, and so do the
    transitions out of node M (MD, MI, II, DD) as at a model's end."""
    def node_order(a, Q8):                     # [..., Q8, 8] -> [..., 8*Q8] by node
        return np.swapaxes(a, -1, -2).reshape(a.shape[:-2] + (8 * Q8,))

    def striped(a, Q8):                        # inverse of node_order
        return np.swapaxes(a.reshape(a.shape[:-1] + (8, Q8)), -1, -2)

    Q0, Q8 = vp.Q8, max(2, (M - 1) // 8 + 1)
    tr = np.full((8, 8 * Q8), -32768, np.int16)
    t0 = np.concatenate([vp.twv[:7 * Q0].reshape(Q0, 7, 8).transpose(1, 0, 2), vp.twv[7 * Q0:][None]])
    tr[:, :M] = node_order(t0, Q0)[:, :M]
    tr[4:, M - 1] = -32768
    tq = striped(tr, Q8)                       # [8, Q8, 8]
    twv = np.concatenate([tq[:7].transpose(1, 0, 2).reshape(7 * Q8, 8), tq[7]])
    rw = np.full((vp.Kp, 8 * Q8), -32768, np.int16)
    rw[:, :M] = node_order(vp.rwv, Q0)[:, :M]
    return F.VProfile(M, np.ascontiguousarray(twv), np.ascontiguousarray(striped(rw, Q8)), vp.xw, vp.scale_w,
                      vp.nj, vp.base_w, vp.ddbound_w)

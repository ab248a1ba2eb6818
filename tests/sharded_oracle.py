"""Test double for one rank's block of a split Jacobi BP sweep: the FP64
oracle (``oracle/bp_oracle.py``) on the block's local network, with the same
interface as ``gbtn.sharded.GpuShard``.  Test infrastructure only."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import bp_oracle as O  # noqa: E402


class OracleShard:
    def __init__(self, plan):
        self.plan = plan
        t = plan.local
        self.g = O.Graph(t.nv, t.edges, t.site_dims, t.edge_dims, legs=[list(l) for l in t.legs])
        self.A = [np.asarray(x, dtype=np.float64) for x in t.tensors]
        self.msgs = None

    def init_messages(self, kind="identity"):
        self.msgs = O.identity_messages(self.g) if kind == "identity" else O.ones_messages(self.g)

    def sweep(self, want_diff):
        new, _, _ = O.bp_update(self.g, self.A, self.msgs, maxiter=1, schedule="parallel")
        diffs = np.array([O.message_diff(new[de], self.msgs[de]) for de in range(2 * self.g.ne)])
        self.msgs = new
        return diffs if want_diff else None

    def get_messages(self):
        return O.flatten_messages(self.g, self.msgs)

    def set_messages(self, flat):
        self.msgs = O.unflatten_messages(self.g, np.asarray(flat))

    def close(self):
        pass

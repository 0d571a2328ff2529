"""One photon's state (excalibur/photon/photon.py:5-78).

The null-condition diagnostics evaluate the metric on the GPU
(`exc_null_error`, `exc_metric_tensor`).
"""
import numpy as np

from .photon_history import PhotonHistory


class Photon:
    def __init__(self, position, direction, weight=1.0):
        self.x = np.asarray(position, dtype=float)
        self.u = np.asarray(direction, dtype=float)
        self.quantities = np.array([])
        self.weight = weight
        self.history = PhotonHistory()

    def null_condition(self, metric):
        """g_{mu nu} u^mu u^nu (diagonal metrics)."""
        g = metric.metric_tensor(self.x)
        return float(np.dot(self.u, np.dot(g, self.u)))

    def null_condition_relative_error(self, metric, *, debug: bool = False):
        """|g u u| / (|g00 u0^2| + sum_i |g_ii u_i^2|) (photon.py:46-68), on the GPU."""
        from .._evaluate import null_error

        rel, st = null_error(metric, np.concatenate([self.x, self.u]))
        if int(st) != 0:
            raise ValueError("metric evaluation failed at the photon position")
        return float(rel)

    def photon_norm(self, metric):
        return self.null_condition_relative_error(metric)

    def photon_norm_abs(self, metric):
        return float(np.sqrt(abs(self.null_condition(metric))))

    def state_quantities(self, relevant_quantities):
        self.quantities = relevant_quantities(self.x)

    @property
    def state(self):
        return np.concatenate([self.x, self.u, self.quantities])

    def record(self):
        self.history.append(self.state)

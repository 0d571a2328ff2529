"""Metric interface (excalibur/metrics/base_metric.py:5-25)."""
from abc import ABC, abstractmethod


class Metric(ABC):
    @abstractmethod
    def metric_tensor(self, x):
        """Metric tensor at x."""

    @abstractmethod
    def christoffel(self, x):
        """Christoffel symbols Gamma^mu_{nu sigma} as a [4, 4, 4] array."""

    @abstractmethod
    def geodesic_equations(self, state):
        """d/dlambda [x^mu, u^mu]."""

    @abstractmethod
    def metric_physical_quantities(self, state):
        """Quantities recorded with each trajectory row."""

    @abstractmethod
    def descriptor(self, device, split=False):
        """The C ABI ExcMetric for this spacetime (see trace.MetricDescriptor)."""

"""Observables from photon trajectories (excalibur/observables/__init__.py): the redshift
components; the plotting helpers of the reference are not part of this package."""

from .redshift import RedshiftCalculator, compute_redshift_components, compute_total_redshift

__all__ = ["compute_redshift_components", "compute_total_redshift", "RedshiftCalculator"]

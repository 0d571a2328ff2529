"""GB300-native backward photon-geodesic tracer (drop-in for excalibur's hot path).

The reference's classes keep their names and signatures:
  core.cosmology.LCDM_Cosmology / StaticCosmology, grid.grid.Grid,
  grid.interpolator_4d_fast.InterpolatorFast, metrics.*_fast, integration.integrator.Integrator,
  photon.photon.Photon, photon.photons.Photons, observables.redshift.RedshiftCalculator.
Every physics evaluation runs in libexcalibur_gb300.so on the GPU.
"""
__version__ = "0.1.0"

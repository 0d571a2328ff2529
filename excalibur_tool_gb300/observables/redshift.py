"""Redshift decomposition of a recorded trajectory (excalibur/observables/redshift.py:73-424).

Same class and method names as the reference, operating on a recorded
trajectory array (rows [eta, x, y, z, u0..u3, a, Phi, dPhi/dx, dPhi/dy,
dPhi/dz, dPhi/deta]). This is post-processing of records on the host; the
tracer itself produces the same components per photon in place
(observables.lensing.redshift_components).
"""
import numpy as np

from ..core.constants import c


def _simpson(y, x):
    from scipy.integrate import simpson

    return simpson(y, x=x)


class RedshiftCalculator:
    def __init__(self, trajectory, a_of_eta=None, potential_func=None, velocity_func=None):
        self.trajectory = np.asarray(trajectory)
        self.velocity_func = velocity_func
        self.has_quantities = self.trajectory.shape[1] >= 14
        if self.has_quantities:
            self.a_array = self.trajectory[:, 8]
            self.phi_array = self.trajectory[:, 9]
            self.grad_phi_array = self.trajectory[:, 10:13]
            self.phi_dot_array = self.trajectory[:, 13]
            self.a_of_eta = None
            self.potential_func = None
        else:
            if a_of_eta is None or potential_func is None:
                raise ValueError("trajectory has no quantities (shape[1] < 14), so a_of_eta and "
                                 "potential_func must be provided as callables")
            self.a_of_eta = a_of_eta
            self.potential_func = potential_func
        tr = self.trajectory
        self.eta_obs, self.eta_em = tr[0, 0], tr[-1, 0]
        self.x_obs, self.x_em = tr[0, 1:4], tr[-1, 1:4]
        if self.has_quantities:
            self.a_obs, self.a_em = self.a_array[0], self.a_array[-1]
        else:
            self.a_obs, self.a_em = a_of_eta(self.eta_obs), a_of_eta(self.eta_em)

    def compute_homogeneous_redshift(self):
        return (self.a_obs / self.a_em) - 1.0

    def compute_potential_at_endpoints(self):
        if self.has_quantities:
            return self.phi_array[0], self.phi_array[-1]
        return (self.potential_func(*self.x_obs, self.eta_obs), self.potential_func(*self.x_em, self.eta_em))

    def compute_sachs_wolfe_redshift(self):
        p_obs, p_em = self.compute_potential_at_endpoints()
        return (p_obs - p_em) / c ** 2, p_obs, p_em

    def compute_integrated_sachs_wolfe_redshift(self):
        eta = self.trajectory[:, 0]
        if self.has_quantities:
            dphi = self.phi_dot_array * (c ** 2)
        else:
            phi = np.array([self.potential_func(x, y, z, e) for x, y, z, e in
                            zip(self.trajectory[:, 1], self.trajectory[:, 2], self.trajectory[:, 3], eta)])
            dphi = np.gradient(phi, eta)
        return -_simpson(dphi, eta) / c ** 2, dphi

    def compute_doppler_redshift(self):
        if self.velocity_func is None:
            return 0.0, np.zeros(3), np.zeros(3)
        v_obs = self.velocity_func(*self.x_obs, self.eta_obs)
        v_em = self.velocity_func(*self.x_em, self.eta_em)
        disp = self.x_em - self.x_obs
        n_hat = disp / np.linalg.norm(disp)
        return (np.dot(v_obs, n_hat) - np.dot(v_em, n_hat)) / c, v_obs, v_em

    def compute_velocity_gradient_redshift(self):
        return 0.0

    def compute_all_components(self, verbose=False):
        r = {}
        z_H = self.compute_homogeneous_redshift()
        z_SW, p_obs, p_em = self.compute_sachs_wolfe_redshift()
        z_ISW, dphi = self.compute_integrated_sachs_wolfe_redshift()
        z_D, v_obs, v_em = self.compute_doppler_redshift()
        z_v = self.compute_velocity_gradient_redshift()
        r.update(z_H=z_H, z_SW=z_SW, Phi_obs=p_obs, Phi_em=p_em, z_ISW=z_ISW, dPhi_deta_array=dphi, z_D=z_D,
                 v_obs=v_obs, v_em=v_em, z_v=z_v)
        r["z_total"] = z_H + z_SW + z_ISW + z_D + z_v
        r["z_total_exact"] = (1 + z_H) * (1 + z_SW) * (1 + z_ISW) * (1 + z_D) * (1 + z_v) - 1.0
        r["a_obs"], r["a_em"] = self.a_obs, self.a_em
        if verbose:
            print(f"z_H={z_H:.6e} z_SW={z_SW:.6e} z_ISW={z_ISW:.6e} z_total={r['z_total']:.6e}")
        return r


def compute_redshift_components(trajectory, a_of_eta, potential_func, velocity_func=None, verbose=False):
    return RedshiftCalculator(trajectory, a_of_eta, potential_func, velocity_func).compute_all_components(verbose)


def compute_total_redshift(trajectory, a_of_eta, potential_func, velocity_func=None):
    """z_total of compute_redshift_components (redshift.py:454-479)."""
    return compute_redshift_components(trajectory, a_of_eta, potential_func, velocity_func, verbose=False)["z_total"]

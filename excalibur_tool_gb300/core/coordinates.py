"""Coordinate conversions used to set up Schwarzschild states.

Same formulas as excalibur/core/coordinates.py:8-133 (spherical <->
cartesian positions and velocities, isotropic radius). These run once per
photon on its initial condition, on the host, exactly as in the reference.
"""
import numpy as np


def spherical_to_cartesian(r, theta, phi):
    x = r * np.sin(theta) * np.cos(phi)
    y = r * np.sin(theta) * np.sin(phi)
    z = r * np.cos(theta)
    return x, y, z


def cartesian_to_spherical(x, y, z):
    r = np.sqrt(x ** 2 + y ** 2 + z ** 2)
    theta = np.arccos(z / r)
    phi = np.arctan2(y, x)
    return r, theta, phi


def cartesian_velocity_to_spherical(x, y, z, vx, vy, vz):
    r, theta, phi = cartesian_to_spherical(x, y, z)
    vr = (x * vx + y * vy + z * vz) / r
    vtheta = ((z * (x * vx + y * vy) - (x ** 2 + y ** 2) * vz)) / (r ** 2 * np.sqrt(x ** 2 + y ** 2))
    vphi = (x * vy - y * vx) / (x ** 2 + y ** 2)
    return vr, vtheta, vphi


def spherical_to_isotropic_radius(r_spherical, r_s):
    b = r_s / 2
    c = (r_s ** 2) / 16 - r_spherical
    disc = b ** 2 - 4 * c
    if np.any(disc < 0):
        raise ValueError("No real solution for isotropic radius.")
    return (-b + np.sqrt(disc)) / 2


def isotropic_to_spherical_radius(r_isotropic, r_s):
    return r_isotropic * (1 + r_s / (4 * r_isotropic)) ** 2


def cartesian_to_isotropic_radius(x, y, z, center, r_s):
    r = np.sqrt((x - center[0]) ** 2 + (y - center[1]) ** 2 + (z - center[2]) ** 2)
    return spherical_to_isotropic_radius(r, r_s)

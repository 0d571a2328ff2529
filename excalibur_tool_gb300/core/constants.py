"""SI constants used by the tracer.

Values are the ones the reference hard-wires for its SI unit system
(excalibur/core/constants.py:7-16, selected at :22-35); they are physical
constants and must be identical for the traced numbers to agree. Only the SI
system is supported (the reference's "natural" branch overwrites one_Mpc
with a year, constants.py:54,58).
"""

c = 299792458                       # speed of light [m/s] (an int, as in the reference)
G = 6.67430e-11                     # [m^3 kg^-1 s^-2]
one_Msun = 1.98847e30               # [kg]
one_pc = 3.085677581e16             # [m]
one_kpc = 1e3 * one_pc
one_Mpc = 1e6 * one_pc
one_Gpc = 1e9 * one_pc
one_yr = 365.25 * 24 * 3600         # [s]
one_Myr = 1e6 * one_yr
one_Gyr = 1e9 * one_yr

# The reference evaluates c**2 and c**4 on Python ints (exact) and converts
# them to float64 at the point of use; these are those correctly-rounded values.
C_F64 = float(c)
C2_F64 = float(c ** 2)
C4_F64 = float(c ** 4)

unit_system = "si"

# the reference's SI names (constants.py:7-16); with the SI system selected they are the values above
c_si, G_si, one_Msun_si, one_pc_si = c, G, one_Msun, one_pc
one_kpc_si, one_Mpc_si, one_Gpc_si = one_kpc, one_Mpc, one_Gpc
one_yr_si, one_Myr_si, one_Gyr_si = one_yr, one_Myr, one_Gyr

"""Physical constants shared by the package (values as pibronic/constants.py:15-50)."""
import numpy as np

#: joules per electron-volt (constants.py:15)
nist_j_per_ev = np.float64(1.6021766208e-19)
#: Boltzmann constant in eV / K (constants.py:24)
boltzman = np.float64(1.38064852e-23) / nist_j_per_ev
#: hbar in the model's units (constants.py:26)
hbar = 1.0
#: default absolute beta step of the finite differences, 1/eV (constants.py:28)
delta_beta = 2.0e-4


def beta(temperature):
    """beta = 1 / (kB T) in 1/eV for T in Kelvin (constants.py:41-44)."""
    return 1.0 / (temperature * boltzman)


def extract_T_from_beta(b):
    """Temperature in Kelvin for a beta in 1/eV (constants.py:47-50)."""
    return 1.0 / (b * boltzman)

"""Physical constants (src/dftpy/constants.py:66-97).

Bohr (Angstrom) and Hartree (eV) are the CODATA-2014 values ASE derives,
so recpot files (eV*A^3, A^-1) convert exactly as the reference converts them.
"""
import math

_e, _me, _hp = 1.6021766208e-19, 9.10938356e-31, 6.626070040e-34
_eps0 = 1.0 / (4.0e-7 * math.pi) / 299792458.0 ** 2
_hbar = _hp / (2.0 * math.pi)

BOHR = 4.0e10 * math.pi * _eps0 * _hbar ** 2 / _me / _e ** 2      # Angstrom
HARTREE = _me * _e ** 3 / 16.0 / math.pi ** 2 / _eps0 ** 2 / _hbar ** 2  # eV

C_TF = 2.87123400018819181594
TKF0 = 6.18733545256027186194
CBRT_TWO = 1.25992104989487316477
ZERO = 1e-30

LEN_CONV = {"Angstrom": {"Bohr": 1.0 / BOHR, "Angstrom": 1.0}, "Bohr": {"Angstrom": BOHR, "Bohr": 1.0}}
ENERGY_CONV = {"Hartree": {"eV": HARTREE, "Hartree": 1.0}, "eV": {"Hartree": 1.0 / HARTREE, "eV": 1.0}}
# ase.units: GPa = 1e9 J/m^3 in eV/Angstrom^3 (J = 1/e eV, m = 1e10 Angstrom)
GPA = 1e9 / _e / 1e30
FORCE_CONV = {"Ha/Bohr": {"eV/A": HARTREE / BOHR, "Ha/Bohr": 1.0}, "eV/A": {"Ha/Bohr": BOHR / HARTREE, "eV/A": 1.0}}
STRESS_CONV = {"Ha/Bohr3": {"eV/A3": HARTREE / BOHR ** 3, "GPa": HARTREE / BOHR ** 3 / GPA, "Ha/Bohr3": 1.0},
               "eV/A3": {"Ha/Bohr3": BOHR ** 3 / HARTREE, "GPa": 1.0 / GPA, "eV/A3": 1.0}}

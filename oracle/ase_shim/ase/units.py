"""Physical constants in ASE's unit system (eV, Angstrom), CODATA 2014.

Test infrastructure only: this is a stand-in for the ``ase.units`` module so
that the reference DFTpy sources can be imported in a container without ASE
(reference: src/dftpy/constants.py:3 imports ``ase.units``).  Every derived
constant is computed from the CODATA-2014 base constants with the textbook
formulas (Bohr radius 4*pi*eps0*hbar^2/(m_e e^2), Hartree m_e e^4/(4*pi*eps0*hbar)^2).
The product package uses the same two numbers (Bohr, Hartree) so that recpot
files written here and read there round-trip exactly.
"""
from math import pi, sqrt

_c = 299792458.0
_mu0 = 4.0e-7 * pi
_Grav = 6.67408e-11
_hplanck = 6.626070040e-34
_e = 1.6021766208e-19
_me = 9.10938356e-31
_mp = 1.672621898e-27
_Nav = 6.022140857e23
_k = 1.38064852e-23
_amu = 1.660539040e-27

_eps0 = 1.0 / _mu0 / _c ** 2
_hbar = _hplanck / (2.0 * pi)

Ang = Angstrom = 1.0
nm = 10.0
m = 1.0e10
eV = 1.0
J = 1.0 / _e
kJ = 1000.0 / _e
kcal = 4.184 * kJ
mol = _Nav

Bohr = 4.0e10 * pi * _eps0 * _hbar ** 2 / _me / _e ** 2
Hartree = _me * _e ** 3 / 16.0 / pi ** 2 / _eps0 ** 2 / _hbar ** 2
Ha = Hartree
Rydberg = 0.5 * Hartree
Ry = Rydberg
kB = _k / _e
alpha = _e ** 2 / (4.0 * pi * _eps0) / _hbar / _c

second = 1.0e10 * sqrt(_e / _amu)
s = second
fs = 1.0e-15 * second
kg = 1.0 / _amu
C = 1.0 / _e
A = 1.0 / _e / second
Pascal = (1.0 / _e) / 1.0e30
GPa = 1.0e9 * Pascal
bar = 1.0e5 * Pascal
Debye = 1.0 / 1.0e11 / _e / _c
invcm = 100.0 * _c * _hplanck / _e

_aut = _hbar / (alpha ** 2 * _me * _c ** 2)
_auv = _e ** 2 / _hbar / (4.0 * pi * _eps0)
_aup = alpha * _me * _c
_auf = alpha ** 3 * _me ** 2 * _c ** 3 / _hbar
AUT = second * _aut

"""Derived properties (src/dftpy/properties/potential.py:3-7) on the device."""

__all__ = ["get_electrostatic_potential"]


def get_electrostatic_potential(rho, evaluator):
    """The local pseudopotential plus the Hartree potential of rho, from the
    evaluator's 'PSEUDO' and 'HARTREE' functionals (potential.py:3-7)."""
    vloc = evaluator.funcDict["PSEUDO"]
    vhart = evaluator.funcDict["HARTREE"]
    return vloc(rho, calcType={"V"}).potential + vhart(rho, calcType={"V"}).potential

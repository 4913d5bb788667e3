"""``ase.calculators`` stand-in (test infrastructure only): the package the
reference calculator imports from (src/dftpy/api/api4ase.py:8)."""

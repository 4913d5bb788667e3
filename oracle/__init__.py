"""CPU oracle for the orbital-free DFT E+V hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
package: it is the checker that the CUDA path is compared against in
``tests/``, in ``__graft_entry__.smoke()`` and in ``bench.py``'s CPU-baseline
leg.  ``ofdft_np`` restates the reference algorithm (Quantum-MultiScale/DFTpy,
``src/dftpy/...``) in numpy, function by function, citing the reference line
it follows.  It is pinned against golden vectors produced by the reference
itself (``tests/golden/make_golden.py`` imports the reference with the
``ase_shim`` stand-in and records its outputs).
"""

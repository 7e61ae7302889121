"""CPU oracle for the direct-minimisation energy-and-gradient path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
package: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` use it, and only as the checker (or as the timed CPU
baseline), never as a fallback for the CUDA path.

``restatement.py`` is an FP64 NumPy restatement of jrystal's algorithm for
this path (every function cites the jrystal file:line it follows).  The
reference itself cannot be imported here (it needs jax, jax_xc, optax and
ase, none of which exist on either machine), so the restatement is pinned
against:

* the golden values of ``jrystal/_src/crystal_test.py:25-61`` (diamond.xyz),
* the FFT-versus-direct-sum identity of ``jrystal/_src/pw_test.py:36-49``,
* the energy/potential identities of ``jrystal/_src/energy_test.py:61-112``,
* the Kohn-Sham trace identity of ``jrystal/_src/hamiltonian_test.py:78-102``,
* central finite differences for the hand-written gradient.

The exchange-correlation values (jax_xc 0.0.8 ``lda_x`` + ``lda_c_vwn``) and
the optimiser (optax ``adam``) are restated from their published formulas;
no reference test pins their values, so that part of the parity is unpinned.
"""

"""CPU oracle for the nssDMRG superblock eigensolver path.

Test infrastructure only: this package restates the reference library's
algorithm on the CPU so that the CUDA path can be checked against it.  Only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it, and only as the reference the results are
compared with (or timed against); nothing in the shipped
package ``nssdmrg_gb300`` imports, links or executes anything from here.

Parity pins (checked by ``tests/test_oracle_pins.py``): the reference's own
golden files ``test/src/Spin1d_SU2/energy.check`` (two lowest E/site after one
iDMRG step from the shipped restart blocks, asserted by the reference at 1e-12),
``test/src/Hubbard1d/energy.check`` and ``Sentropy.check``, and the 39-step
from-scratch iDMRG trajectories ``test/src/*/L40.energy.check`` /
``L40.Sentropy.check``, converted into ``tests/golden/*.npz`` by
``tests/golden/make_golden.py``.
"""

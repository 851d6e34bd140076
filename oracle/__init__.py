"""CPU oracle for pyAtmosphere's split-step propagation path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this
package, and only as the checker or as the timed CPU baseline.  The engine in
``pyatmosphere_gb300`` never imports it and has no CPU fallback.

Parity is pinned: ``tests/test_oracle_golden.py`` checks this restatement
against golden vectors produced by running the reference itself
(``tests/golden/make_golden.py``) on identical injected spectra.
"""
from .atm_oracle import *  # noqa: F401,F403

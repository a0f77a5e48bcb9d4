"""Host threads do not change results.

The library runs several host phases of a DMRG step on threads (the
superblock states, sector filters and A x B terms per sector, the staging
copy, the packed sector rows, the renormalisation's extraction and CSR
assembly per operator); each task writes only its own slots.  A whole run
with those loops on threads (default) and on the calling thread alone
(NSS_HOST_THREADS=1, read once per process, hence the subprocesses) must
give bit-identical energies, truncation errors, entropies and kept
dimensions.  The chain is large enough for every threaded loop to take its
parallel branch (superblocks above 200 000 states, device renormalisation
of blocks above 256 states).  The tile tuner is off, so that both runs take
the same H*psi plan.
"""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

SCRIPT = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import nssdmrg_gb300 as nss
d = nss.DMRG(nss.MODEL_HEISENBERG_ONE, 12, 512, dmrg_qn=(0.0, 0.0), lanc_neigen=1)
recs = d.infinite()
d.close()
print(json.dumps([[r["n"], r["energy"][0].hex(), r["trunc_left"].hex(), r["trunc_right"].hex(),
                   r["entropy_left"].hex(), r["entropy_right"].hex(), r["m_left"], r["m_right"]]
                  for r in recs]))
"""


def _run(threads):
    env = dict(os.environ, NSS_TC_AUTO="0")
    env.pop("NSS_HOST_THREADS", None)
    if threads is not None:
        env["NSS_HOST_THREADS"] = str(threads)
    out = subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT)], env=env, capture_output=True, text=True,
                         timeout=900)
    assert out.returncode == 0, out.stderr[-3000:]
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_run_with_host_threads_equals_serial_host_run():
    threaded = _run(None)
    serial = _run(1)
    assert max(r[0] for r in threaded) > 200000      # the largest superblocks take the parallel branches
    assert len(threaded) == len(serial)
    for k, (a, b) in enumerate(zip(threaded, serial)):
        assert a == b, f"step {k}: {a} != {b}"

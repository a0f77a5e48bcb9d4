"""Block restart files through the library's reader and writer (host C++,
the reference's text layout, src/BLOCKS/BLOCKS.f90:418-537).

The reader is pinned by the reference's known-answer test: its length-39
restart blocks (here rewritten from the fixtures in the legacy layout of the
shipped files, old operator names and "sign" type included) loaded into the
driver and advanced by one step give energy.check (asserted at 1e-12 by
spinSU2_1d.f90:246-255 for the spin chain; 1e-6 for the Hubbard chain,
hm_1d.f90:139-147, met here at 1e-12).  The writer is checked by a round
trip: blocks written after a run read back into a new driver and written
again give the same file, the oracle's reader parses it, and the run
continued from them reproduces the energies of an uninterrupted run.
"""
import numpy as np
import pytest

from conftest import load_npz
from oracle.restart_io import parse_block
from tests.golden.blockio import restart_text, unpack_block

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nss():
    import nssdmrg_gb300 as nss
    nss.lib()
    return nss


@pytest.mark.parametrize("name", ["spin", "hubbard"])
def test_reference_restart_blocks_reproduce_energy_check(nss, tmp_path, name):
    z = load_npz(f"kat_{name}.npz")
    ldmrg, mdmrg, neigen = (int(x) for x in z["params"])
    paths = []
    for side in ("left", "right"):
        p = tmp_path / f"block_{side}.restart"
        p.write_text(restart_text(unpack_block(side, z), legacy=True))
        paths.append(p)
    if name == "spin":
        d = nss.DMRG(0, ldmrg, mdmrg, dmrg_qn=(0.0, 0.0), lanc_neigen=neigen, lanc_tolerance=1e-12)
    else:
        d = nss.DMRG(2, ldmrg, mdmrg, u=0.0, hfmode=True, dmrg_qn=(0.5, 0.5), lanc_neigen=neigen,
                     lanc_tolerance=1e-12)
    d.load_blocks(*paths)
    recs = d.infinite()
    assert len(recs) == 1 and recs[0]["left_length"] == ldmrg
    e = np.array(recs[0]["energy"][:neigen])
    np.testing.assert_allclose(e, z["golden_energy"][:neigen], rtol=1e-12, atol=0)


def test_written_blocks_round_trip_and_continue(nss, tmp_path):
    """Spin-1/2 chain, M=24: an infinite run to length 9 ends on its
    enlarged, unrenormalised blocks; they are saved, read back into a new
    driver and written again (the same file), parsed by the oracle's reader,
    and the new driver continues the infinite algorithm from them to length
    12.  Its first superblock contains the uninterrupted run's (that run had
    truncated the length-9 blocks), so its energy is at most that run's; by
    length 12 the two agree to the truncation level."""
    def mk(ld):
        return nss.DMRG(0, ld, 24, dmrg_qn=(0.0, 0.0), lanc_neigen=1, lanc_tolerance=1e-12, save_umat=True)

    full = {r["left_length"]: r["energy"][0] for r in mk(12).infinite()}
    short = mk(9)
    short.infinite()
    l1, r1 = tmp_path / "l1.restart", tmp_path / "r1.restart"
    short.save_blocks(l1, r1)
    b = parse_block(l1.read_text())
    assert b.length == 9 and list(b.ops) == ["H", "S_z_n", "S_p_n"]
    c = mk(12)
    c.load_blocks(l1, r1)
    l2, r2 = tmp_path / "l2.restart", tmp_path / "r2.restart"
    c.save_blocks(l2, r2)
    assert l1.read_text() == l2.read_text() and r1.read_text() == r2.read_text()
    recs = c.infinite()
    assert [r["left_length"] for r in recs] == [10, 11, 12]
    assert recs[0]["energy"][0] <= full[10] + 1e-12
    assert abs(recs[-1]["energy"][0] - full[12]) < 1e-6


def test_load_rejects_other_models(nss, tmp_path):
    z = load_npz("kat_hubbard.npz")
    p = tmp_path / "h.restart"
    p.write_text(restart_text(unpack_block("left", z)))
    d = nss.DMRG(0, 40, 20, dmrg_qn=(0.0, 0.0), lanc_neigen=1)
    with pytest.raises(nss.NssError):
        d.load_blocks(p, None)
    with pytest.raises(nss.NssError):
        d.load_blocks(tmp_path / "missing.restart", None)

"""The library's restart-file reader and writer (host C++), on CPU.

The fixtures' blocks (read from the reference's restart files by the
oracle's reader) are written in the shipped files' legacy layout by the
test-side writer, read and rewritten by the library, and parsed again by
the oracle's reader: the block must come back exactly, under the current
operator names; rewriting the library's own output reproduces it byte for
byte."""
import numpy as np
import pytest

import nssdmrg_gb300 as nss
from conftest import load_npz
from oracle.restart_io import parse_block
from tests.golden.blockio import restart_text, unpack_block


@pytest.mark.parametrize("name", ["spin", "hubbard"])
def test_rewrite_round_trips(tmp_path, name):
    z = load_npz(f"kat_{name}.npz")
    for side in ("left", "right"):
        b = unpack_block(side, z)
        src, out, out2 = tmp_path / "in.restart", tmp_path / "out.restart", tmp_path / "out2.restart"
        src.write_text(restart_text(b, legacy=True))
        nss.restart_rewrite(src, out)
        r = parse_block(out.read_text())
        assert (r.length, r.dim, r.sitetype) == (b.length, b.dim, b.sitetype)
        np.testing.assert_array_equal(r.basis, b.basis)
        assert list(r.ops) == list(b.ops)
        for k in b.ops:
            assert r.ops[k][1] == b.ops[k][1]
            assert (r.op(k) != b.op(k)).nnz == 0
        nss.restart_rewrite(out, out2)
        assert out.read_text() == out2.read_text()


def test_rewrite_rejects_broken_files(tmp_path):
    bad = tmp_path / "bad.restart"
    bad.write_text(" 3\n 2\n SPIN\n S\n 1\n 1\n 1\n 1\n 0.5\n 1\n 1\n")   # sectors do not cover the basis
    with pytest.raises(nss.NssError):
        nss.restart_rewrite(bad, tmp_path / "x.restart")
    with pytest.raises(nss.NssError):
        nss.restart_rewrite(tmp_path / "missing.restart", tmp_path / "y.restart")

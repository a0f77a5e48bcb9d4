"""Reader for the reference's block restart text format (oracle; test only).

Follows read_block (src/BLOCKS/BLOCKS.f90:471-537): length, Dim, SiteType,
OpName, number of sector lists, each sector list (read_sectors_list,
src/LIST/LIST_SECTORS.f90:671-705: size, qdim, then per sector DimQn, qn,
DimMap, map), the operator list (read_operators_list,
src/LIST/LIST_OPERATORS.f90:636-667: size, then key, type and a sparse matrix
per entry) and the rotation-matrix list in the same format.  A sparse matrix
is sp_read_matrix (src/MATRIX/MATRIX_SPARSE.f90:732-770): Nrow Ncol, then per
row its size followed by (col, val) pairs.  All records are Fortran
list-directed, so a whitespace token stream reads them.

The restart files shipped with the reference's tests were written by an
older revision that named operators without the link suffix ("S_z", "C_l1_s1",
"P") and typed the sign operator "sign".  The current code looks them up as
"S_z_n", "C_l1_s1_n", "P_n" with type "psign" (src/DMRG_CONNECT.f90:117-146,
src/BLOCKS/SITES.f90:335-339, :424-431), so the reader maps the legacy names.
"""
from __future__ import annotations

import re

import numpy as np
import scipy.sparse as sp

from .dmrg_oracle import Block, Sectors


class _Tokens:
    def __init__(self, text: str):
        self.tok = text.split()
        self.i = 0

    def next(self) -> str:
        t = self.tok[self.i]
        self.i += 1
        return t

    def int(self) -> int:
        return int(self.next())

    def float(self) -> float:
        return float(self.next().replace("D", "E").replace("d", "e"))


def _read_matrix(t: _Tokens) -> sp.csr_matrix:
    nrow, ncol = t.int(), t.int()
    rows, cols, vals = [], [], []
    for r in range(nrow):
        n = t.int()
        for _ in range(n):
            cols.append(t.int() - 1)
            vals.append(t.float())
            rows.append(r)
    return sp.csr_matrix((np.asarray(vals, float), (np.asarray(rows, int), np.asarray(cols, int))),
                         shape=(nrow, ncol))


_LEGACY = re.compile(r"^(S_z|S_p|P|C_l\d+_s\d+)$")


def _legacy_key(key: str) -> str:
    return key + "_n" if _LEGACY.match(key) else key


def parse_block(text: str) -> Block:
    t = _Tokens(text)
    length = t.int()
    dim = t.int()
    sitetype = t.next().lower()
    _opname = t.next()
    nlists = t.int()
    if nlists != 1:
        raise ValueError("only one sector list per block is supported")
    size, qdim = t.int(), t.int()
    basis = np.full((dim, qdim), np.nan)
    for _ in range(size):
        dq = t.int()
        qn = [t.float() for _ in range(dq)]
        nmap = t.int()
        for _ in range(nmap):
            basis[t.int() - 1, :] = qn
    if np.isnan(basis).any():
        raise ValueError("restart sectors do not cover the block basis")
    nops = t.int()
    ops = {}
    for _ in range(nops):
        key = _legacy_key(t.next())
        typ = t.next()
        if typ == "none":
            typ = ""
        if typ == "sign":
            typ = "psign"
        ops[key] = (_read_matrix(t), typ)
    sitetype = "spin" if sitetype.startswith("s") else "fermion"
    blk = Block(length, dim, sitetype, basis, ops)
    # assignment through the block constructor rebuilds the sector list from
    # the basis (equality_sector_list, src/LIST/LIST_SECTORS.f90:507-519)
    Sectors(basis)
    return blk


def read_block(path: str) -> Block:
    with open(path) as f:
        return parse_block(f.read())

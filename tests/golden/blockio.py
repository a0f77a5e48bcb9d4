"""(De)serialisation of oracle blocks to the npz fixtures of this folder."""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from oracle.dmrg_oracle import Block


def pack_block(prefix: str, blk: Block, out: dict):
    out[f"{prefix}/meta"] = np.array([blk.length, blk.dim, 1 if blk.sitetype == "fermion" else 0])
    out[f"{prefix}/basis"] = blk.basis
    out[f"{prefix}/keys"] = np.array([k for k in blk.ops])
    out[f"{prefix}/types"] = np.array([blk.ops[k][1] for k in blk.ops])
    for k, (m, _) in blk.ops.items():
        m = m.tocsr()
        out[f"{prefix}/{k}/indptr"] = m.indptr.astype(np.int32)
        out[f"{prefix}/{k}/indices"] = m.indices.astype(np.int32)
        out[f"{prefix}/{k}/data"] = m.data
        out[f"{prefix}/{k}/shape"] = np.array(m.shape)


def unpack_block(prefix: str, z) -> Block:
    length, dim, ferm = (int(x) for x in z[f"{prefix}/meta"])
    ops = {}
    for k, t in zip(z[f"{prefix}/keys"], z[f"{prefix}/types"]):
        k, t = str(k), str(t)
        m = sp.csr_matrix((z[f"{prefix}/{k}/data"], z[f"{prefix}/{k}/indices"], z[f"{prefix}/{k}/indptr"]),
                          shape=tuple(z[f"{prefix}/{k}/shape"]))
        ops[k] = (m, t)
    return Block(length, dim, "fermion" if ferm else "spin", np.asarray(z[f"{prefix}/basis"], float), ops)


_LEGACY_NAMES = {"S_z_n": "S_z", "S_p_n": "S_p", "P_n": "P", "C_l1_s1_n": "C_l1_s1", "C_l1_s2_n": "C_l1_s2"}


def restart_text(blk: Block, legacy: bool = False) -> str:
    """An oracle block in the reference's restart text layout (write_block,
    src/BLOCKS/BLOCKS.f90:418-447; sectors, operators and matrices as
    src/LIST/LIST_SECTORS.f90:639-669, src/LIST/LIST_OPERATORS.f90:602-631,
    src/MATRIX/MATRIX_SPARSE.f90:703-728), for feeding blocks from these
    fixtures to the library's reader.  legacy: the operator names and sign
    type of the restart files shipped with the reference's tests."""
    out = [f" {blk.length}", f" {blk.dim}", " FERMION" if blk.sitetype == "fermion" else " SPIN",
           " C" if blk.sitetype == "fermion" else " S", " 1"]
    qns, maps = [], []
    for i, q in enumerate(map(tuple, blk.basis)):
        if q not in qns:
            qns.append(q)
            maps.append([])
        maps[qns.index(q)].append(i + 1)
    out += [f" {len(qns)}", f" {blk.basis.shape[1]}"]
    for q, m in zip(qns, maps):
        out += [f" {len(q)}", " " + " ".join(repr(float(x)) for x in q), f" {len(m)}", " " + " ".join(map(str, m))]
    out.append(f" {len(blk.ops)}")
    for k, (m, t) in blk.ops.items():
        if legacy:
            k = _LEGACY_NAMES.get(k, k)
            t = "sign" if t == "psign" else t
        out += [f" {k}", f" {t or 'none'}"]
        m = sp.csr_matrix(m)
        out.append(f" {m.shape[0]} {m.shape[1]}")
        for i in range(m.shape[0]):
            out.append(f" {m.indptr[i + 1] - m.indptr[i]}")
            for p in range(m.indptr[i], m.indptr[i + 1]):
                out.append(f" {m.indices[p] + 1} {float(m.data[p])!r}")
    out.append(" 0")
    return "\n".join(out) + "\n"

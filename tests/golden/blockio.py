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

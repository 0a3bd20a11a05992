"""Oracle of the topology build — TEST INFRASTRUCTURE ONLY.

Restates, with numpy, the arrays the library derives from a triangle and a
hinge list: the BSR pattern of MDK (node pairs sharing a triangle or a
hinge, columns ascending within a row), the element contributions of every
block in the order the reference inserts its triplets (Forces.cpp:331-930:
faces in order, each with its 3x3 (row vertex, column vertex) blocks, then
hinges in order with their 4x4; setFromTriplets sums duplicates in that
order, Forces.cpp:925-929), and each node's faces in order.  Contribution
code: element << 7 | hinge << 6 | row vertex << 3 | column vertex; face
entry: face << 2 | local vertex.
"""
import numpy as np


def build(n_nodes, tri, hinge):
    tri = np.asarray(tri, np.int64).reshape(-1, 3)
    hinge = np.asarray(hinge, np.int64).reshape(-1, 4)
    T, H = len(tri), len(hinge)
    # one record per (element, row vertex, column vertex), insertion order
    ta, tb = np.meshgrid(np.arange(3), np.arange(3), indexing="ij")
    ha, hb = np.meshgrid(np.arange(4), np.arange(4), indexing="ij")
    rows = np.concatenate([tri[:, ta.ravel()].ravel(), hinge[:, ha.ravel()].ravel()])
    cols = np.concatenate([tri[:, tb.ravel()].ravel(), hinge[:, hb.ravel()].ravel()])
    codes = np.concatenate([
        (np.arange(T)[:, None] << 7 | ta.ravel()[None, :] << 3 | tb.ravel()[None, :]).ravel(),
        (np.arange(H)[:, None] << 7 | 64 | ha.ravel()[None, :] << 3 | hb.ravel()[None, :]).ravel()])
    seq = np.arange(len(rows))
    order = np.lexsort((seq, cols, rows))  # stable in insertion order per block
    r, c, code = rows[order], cols[order], codes[order]
    new = np.ones(len(r), bool)
    new[1:] = (r[1:] != r[:-1]) | (c[1:] != c[:-1])
    starts = np.nonzero(new)[0]
    colidx = c[starts].astype(np.int32)
    blk_row = r[starts]
    rowptr = np.zeros(n_nodes + 1, np.int64)
    np.add.at(rowptr, blk_row + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    cptr = np.append(starts, len(r)).astype(np.int32)
    # node -> faces, in face order
    fnode = tri.ravel()
    fcode = (np.arange(T)[:, None] << 2 | np.arange(3)[None, :]).ravel()
    o = np.lexsort((fcode, fnode))
    nf_ptr = np.zeros(n_nodes + 1, np.int64)
    np.add.at(nf_ptr, fnode + 1, 1)
    return dict(rowptr=rowptr, colidx=colidx, cptr=cptr, contrib=code.astype(np.int32),
                nf_ptr=np.cumsum(nf_ptr).astype(np.int32), nf_list=fcode[o].astype(np.int32))

"""CPU reference of the learned preconditioner's network and probe loss.

TEST INFRASTRUCTURE ONLY: checks the library's hand-written CUDA forward and
backward kernels (eol-cloth_gb300/csrc/learned.cu).  The same network, the
same BF16 rounding of the weight matrices in the forward pass (biases stay
FP32; straight-through in the backward pass), the same G assembly and the
same probe loss, written with torch on the CPU in FP64 and differentiated by
torch.autograd.
"""
import numpy as np
import torch

H, FN, FE, OE, ON, LAYERS = 64, 8, 9, 18, 3, 3
EDGE_IN = 2 * H + FE


def layout():
    o = 0
    L = {}
    def take(name, n):
        nonlocal o
        L[name] = (o, n)
        o += n
    take("Wn", FN * H); take("bn", H)
    take("Wg", FE * H); take("bg", H)
    for l in range(LAYERS):
        take("W%d" % l, 2 * H * H); take("b%d" % l, H)
    take("Wt", H * ON); take("bt", ON)
    take("Wo", EDGE_IN * OE); take("bo", OE)
    return L, o


def bf16_round(t):
    return t.to(torch.bfloat16).to(t.dtype)


def graph(rowptr, colidx):
    """Edges (i < j) in pattern order, their block positions, incidence."""
    n = len(rowptr) - 1
    pos = {}
    for i in range(n):
        for k in range(rowptr[i], rowptr[i + 1]):
            pos[(i, int(colidx[k]))] = k
    ei, ej, bij, bji = [], [], [], []
    for i in range(n):
        for k in range(rowptr[i], rowptr[i + 1]):
            j = int(colidx[k])
            if j > i:
                ei.append(i); ej.append(j); bij.append(k); bji.append(pos[(j, i)])
    diag = np.array([pos[(i, i)] for i in range(n)])
    return np.array(ei), np.array(ej), np.array(bij), np.array(bji), diag


def _forward(th, A, rowptr, colidx, pinned):
    """G (nb, 3, 3) from the FP64 parameter vector th: weight matrices are
    rounded to BF16 (straight-through for the gradient), biases are not —
    as in the library's kernels."""
    L, P = layout()
    n = len(rowptr) - 1
    ei, ej, bij, bji, diag = graph(rowptr, colidx)
    m = len(ei)
    A = torch.tensor(np.asarray(A, np.float64).reshape(-1, 3, 3))
    pin = torch.tensor(np.asarray(pinned, bool).reshape(n, 3))
    free = (~pin).double()

    def W(name, shape):
        o, c = L[name]
        v = th[o:o + c]
        if name.startswith("W"):
            v = v + (bf16_round(v) - v).detach()
        return v.reshape(shape)

    D = A[diag]
    d = torch.stack([D[:, 0, 0], D[:, 1, 1], D[:, 2, 2]], 1)
    mdiag = d.mean(1)
    # node features
    blk_norm = torch.sqrt((A ** 2).sum((1, 2)))
    row_of = np.repeat(np.arange(n), np.diff(rowptr))
    off = torch.zeros(n, dtype=torch.float64).index_add(
        0, torch.tensor(row_of), torch.where(torch.tensor(np.arange(len(row_of)) != diag[row_of]),
                                             blk_norm, torch.zeros_like(blk_norm)))
    dn = torch.sqrt((D ** 2).sum((1, 2)))
    fN = torch.stack([torch.log(1e-12 + off / dn), D[:, 0, 0] / mdiag, D[:, 1, 1] / mdiag,
                      D[:, 2, 2] / mdiag, D[:, 0, 1] / mdiag, D[:, 0, 2] / mdiag,
                      D[:, 1, 2] / mdiag, pin.double().mean(1)], 1)
    sc = 1.0 / torch.sqrt(mdiag[ei] * mdiag[ej])
    fE = A[bij].reshape(m, 9) * sc[:, None]
    relu = torch.relu
    h = relu(fN @ W("Wn", (FN, H)) + W("bn", (H,)))
    g = torch.sigmoid(fE @ W("Wg", (FE, H)) + W("bg", (H,)))
    deg = torch.zeros(n, dtype=torch.float64).index_add(0, torch.tensor(ei), torch.ones(m, dtype=torch.float64))
    deg = deg.index_add(0, torch.tensor(ej), torch.ones(m, dtype=torch.float64))
    dinv = torch.where(deg > 0, 1.0 / deg, torch.zeros_like(deg))
    tei, tej = torch.tensor(ei), torch.tensor(ej)
    for l in range(LAYERS):
        agg = torch.zeros(n, H, dtype=torch.float64)
        agg = agg.index_add(0, tei, g * h[tej]).index_add(0, tej, g * h[tei]) * dinv[:, None]
        h = relu(torch.cat([h, agg], 1) @ W("W%d" % l, (2 * H, H)) + W("b%d" % l, (H,)))
    theta = h @ W("Wt", (H, ON)) + W("bt", (ON,))
    o = torch.cat([h[tei], h[tej], fE], 1) @ W("Wo", (EDGE_IN, OE)) + W("bo", (OE,))
    Ut = o[:, :9].reshape(m, 3, 3)
    Vt = o[:, 9:].reshape(m, 3, 3)
    s = 1.0 / torch.sqrt(d)
    U = s[tei][:, :, None] * Ut
    V = s[tej][:, :, None] * Vt
    nb = A.shape[0]
    G = torch.zeros(nb, 3, 3, dtype=torch.float64)
    lam = torch.nn.functional.softplus(theta) / d
    G = G.index_add(0, torch.tensor(diag), torch.diag_embed(lam))
    G = G.index_add(0, torch.tensor(diag[ei]), U @ U.transpose(1, 2))
    G = G.index_add(0, torch.tensor(diag[ej]), V @ V.transpose(1, 2))
    G = G.index_add(0, torch.tensor(bij), U @ V.transpose(1, 2))
    G = G.index_add(0, torch.tensor(bji), V @ U.transpose(1, 2))
    # free-DOF mask on both sides
    col_of = torch.tensor(np.asarray(colidx))
    G = G * free[torch.tensor(row_of)][:, :, None] * free[col_of][:, None, :]
    return G, (n, row_of, torch.tensor(np.asarray(colidx)), free, A)


def g_blocks(params, A, rowptr, colidx, pinned):
    """The approximate inverse G (nb x 9, float64) of the network for MDK
    blocks A (nb x 9), BF16 weights, FP64 arithmetic."""
    th = torch.tensor(np.asarray(params, np.float64))
    G, _ = _forward(th, A, rowptr, colidx, pinned)
    return G.detach().numpy().reshape(-1, 9)


def loss_and_grad(params, A, rowptr, colidx, pinned, probes):
    """params: (P,) float32; A: (nb, 9) float32 block values; pinned: (3N,)
    bool; probes: (k, 3N) float32.  Returns (loss, grad (P,) float64)."""
    th = torch.tensor(np.asarray(params, np.float64), requires_grad=True)
    G, (n, row_of, col_of, free, A) = _forward(th, A, rowptr, colidx, pinned)
    loss = 0.0
    k = probes.shape[0]
    At = A
    for q in range(k):
        w = torch.tensor(np.asarray(probes[q], np.float64)).reshape(n, 3)
        y = torch.zeros(n, 3, dtype=torch.float64).index_add(
            0, torch.tensor(row_of), (At @ w[col_of][:, :, None])[:, :, 0])
        z = torch.zeros(n, 3, dtype=torch.float64).index_add(
            0, torch.tensor(row_of), (G @ y[col_of][:, :, None])[:, :, 0])
        r = (z - w) * free
        nrm = ((w * free) ** 2).sum()
        loss = loss + (r ** 2).sum() / (k * nrm)
    loss.backward()
    return float(loss.detach()), th.grad.numpy().astype(np.float64)

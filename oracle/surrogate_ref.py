"""CPU restatement of the learned bond-order surrogate, for the tests only.

Test infrastructure: nothing in the product imports this file.  The
surrogate has no counterpart in the reference; this module states its
mathematics plainly (numpy, float64) so the GPU kernels can be checked:

* descriptors: 16 radial and 16 angular Behler symmetry functions of the
  neighbours within rc (minimum image in a periodic box),
    G2_k = sum_j exp(-eta_r (r_ij - rs_k)^2) fc(r_ij),
    G4_f = 2^(1 - zeta_f) sum_{j<k} (1 + lam_f cos theta_jik)^zeta_f
           exp(-eta_f (r_ij^2 + r_ik^2)) fc(r_ij) fc(r_ik),
    fc(r) = (cos(pi r / rc) + 1) / 2,
  with the parameter table of moleculardynamics_gb300/csrc/md_surrogate.cu
  (default_desc);
* the network 32-64-64-1 (tanh) with the tensor-core roundings of the GPU
  kernels: weights are BF16; in training every operand of a tensor-core
  product (inputs, H1, the two backward deltas and the transposed training
  operands) is rounded to BF16; in inference every A operand is carried as
  a pair of BF16 parts (hi + lo); products accumulate in high precision,
  everything else is FP32/FP64;
* the training loss mean((t - y)^2) and its gradient with respect to the
  parameters, laid out as W1 [64][32], b1 [64], W2 [64][64], b2 [64],
  w3 [64], b3;
* the direct-force head, the second model kind: 32 -> H -> H -> 32 (tanh,
  FP32 on the GPU), parameters W1 [H][32], b1 [H], W2 [H][H], b2 [H],
  W3 [32][H], b3 [32]; its outputs w(x) and the parameter gradient of
  sum_i v_i . w(x_i).
"""
import numpy as np

NDESC, NHID = 32, 64


def bf16(x):
    """Round to BF16 (nearest even) and back, as __float2bfloat16_rn."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def desc_params(rc=3.0):
    d = (rc - 0.8) / 15.0
    rs = 0.8 + d * np.arange(16)
    eta_r = 0.5 / (d * d)
    f = np.arange(16)
    zeta = np.array([1, 2, 4, 16])[f % 4]
    lam = np.where((f // 4) % 2 == 1, -1.0, 1.0)
    eta_a = np.array([0.02, 0.25])[f // 8]
    pref = 2.0 ** (1.0 - zeta)
    return dict(rc=rc, rs=rs, eta_r=eta_r, zeta=zeta, lam=lam, eta_a=eta_a, pref=pref)


def descriptors(pos4, box=None, rc=3.0):
    """(n, 32) descriptors; box = edge of a periodic cube, or None."""
    P = desc_params(rc)
    x = np.asarray(pos4, np.float64)[:, :3]
    n = len(x)
    G = np.zeros((n, NDESC))
    for i in range(n):
        d = x - x[i]
        if box is not None:
            d -= box * np.rint(d / box)
        r = np.sqrt((d * d).sum(1))
        m = (r < rc) & (np.arange(n) != i)
        d, r = d[m], r[m]
        fc = 0.5 * (np.cos(np.pi * r / rc) + 1.0)
        G[i, :16] = (np.exp(-P["eta_r"] * (r[:, None] - P["rs"][None]) ** 2) * fc[:, None]).sum(0)
        S = len(r)
        if S < 2:
            continue
        a, b = np.triu_indices(S, 1)
        c = (d[a] * d[b]).sum(1) / (r[a] * r[b])
        q = r[a] ** 2 + r[b] ** 2
        ff = fc[a] * fc[b]
        base = np.maximum(1.0 + P["lam"][None] * c[:, None], 0.0)
        G[i, 16:] = (P["pref"][None] * base ** P["zeta"][None] *
                     np.exp(-P["eta_a"][None] * q[:, None]) * ff[:, None]).sum(0)
    return G


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + NHID * NDESC].reshape(NHID, NDESC); o += NHID * NDESC
    b1 = p[o:o + NHID]; o += NHID
    W2 = p[o:o + NHID * NHID].reshape(NHID, NHID); o += NHID * NHID
    b2 = p[o:o + NHID]; o += NHID
    w3 = p[o:o + NHID]; o += NHID
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def forward(p, x):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    xb = bf16(x)
    h1 = np.tanh(xb @ bf16(W1).T + b1)
    h2 = np.tanh(bf16(h1) @ bf16(W2).T + b2)
    t = h2 @ w3 + b3
    return t, h1, h2, xb


def split(a):
    """a as the sum of its BF16 rounding and the BF16 rounding of the rest."""
    hi = bf16(a)
    return hi + bf16(np.asarray(a, np.float64) - hi)


def net(p, x):
    """t = net(x) and dt/dx as the inference kernel computes them: every
    tensor-core A operand as a pair of BF16 parts (split), weights BF16."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    h1 = np.tanh(split(x) @ bf16(W1).T + b1)
    h2 = np.tanh(split(h1) @ bf16(W2).T + b2)
    t = h2 @ w3 + b3
    d2 = w3[None] * (1.0 - h2 ** 2)
    dh1 = split(d2) @ bf16(W2)
    d1 = dh1 * (1.0 - h1 ** 2)
    return t, split(d1) @ bf16(W1)


def loss_grad(p, x, y):
    """mean((t - y)^2) and its parameter gradient, as the training kernel."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    n = len(y)
    t, h1, h2, xb = forward(p, x)
    res = t - np.asarray(y, np.float64)
    d3 = 2.0 * res / n
    g_b3 = d3.sum()
    g_w3 = (d3[:, None] * h2).sum(0)
    d2 = d3[:, None] * w3[None] * (1.0 - h2 ** 2)
    g_b2 = d2.sum(0)
    g_W2 = bf16(d2).T @ bf16(h1)
    dh1 = bf16(d2) @ bf16(W2)
    d1 = dh1 * (1.0 - h1 ** 2)
    g_b1 = d1.sum(0)
    g_W1 = bf16(d1).T @ xb
    grad = np.concatenate([g_W1.ravel(), g_b1, g_W2.ravel(), g_b2, g_w3, [g_b3]])
    return float((res ** 2).mean()), grad


def force_grad(p, x, v, rnd=bf16):
    """Gradient over the parameters of sum_i v_i . dt/dx(x_i): the force term
    of the force-matching loss once the loss' sensitivity to dt/dx is the
    direction v.  rnd is the operand rounding (bf16; identity for exact
    arithmetic), applied where the training kernel rounds tensor-core operands."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    xb, vb = rnd(x), rnd(v)
    W1b, W2b = rnd(W1), rnd(W2)
    h1 = np.tanh(xb @ W1b.T + b1)
    zd1 = vb @ W1b.T
    hd1 = (1.0 - h1 ** 2) * zd1
    h2 = np.tanh(rnd(h1) @ W2b.T + b2)
    zd2 = rnd(hd1) @ W2b.T
    hd2 = (1.0 - h2 ** 2) * zd2
    a_zd2 = w3[None] * (1.0 - h2 ** 2)
    a_z2 = w3[None] * (-2.0 * h2 * zd2) * (1.0 - h2 ** 2)
    g_w3 = hd2.sum(0)
    g_b2 = a_z2.sum(0)
    g_W2 = rnd(a_z2).T @ rnd(h1) + rnd(a_zd2).T @ rnd(hd1)
    a_h1 = rnd(a_z2) @ W2b
    a_hd1 = rnd(a_zd2) @ W2b
    a_zd1 = a_hd1 * (1.0 - h1 ** 2)
    a_z1 = (a_h1 + a_hd1 * (-2.0 * h1 * zd1)) * (1.0 - h1 ** 2)
    g_b1 = a_z1.sum(0)
    g_W1 = rnd(a_z1).T @ xb + rnd(a_zd1).T @ vb
    return np.concatenate([g_W1.ravel(), g_b1, g_W2.ravel(), g_b2, g_w3, [0.0]])


def directional(p, x, v):
    """sum_i v_i . dt/dx(x_i) in exact arithmetic (for checking force_grad)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    h1 = np.tanh(x @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    hd1 = (1.0 - h1 ** 2) * (v @ W1.T)
    hd2 = (1.0 - h2 ** 2) * (hd1 @ W2.T)
    return float((hd2 @ w3).sum())


def head_unpack(p, H):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + H * 32].reshape(H, 32); o += H * 32
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + 32 * H].reshape(32, H); o += 32 * H
    b3 = p[o:o + 32]
    return W1, b1, W2, b2, W3, b3


def head_forward(p, x, H):
    """w(x) of the direct-force head (n x 32)."""
    W1, b1, W2, b2, W3, b3 = head_unpack(p, H)
    h1 = np.tanh(np.asarray(x, np.float64) @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ W3.T + b3


def head_grad(p, x, v, H):
    """Parameter gradient of sum_i v_i . w(x_i), in the parameter layout."""
    W1, b1, W2, b2, W3, b3 = head_unpack(p, H)
    x = np.asarray(x, np.float64)
    v = np.asarray(v, np.float64)
    h1 = np.tanh(x @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    d3 = v
    d2 = (d3 @ W3) * (1 - h2 * h2)
    d1 = (d2 @ W2) * (1 - h1 * h1)
    return np.concatenate([(d1.T @ x).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0),
                           (d3.T @ h2).ravel(), d3.sum(0)])

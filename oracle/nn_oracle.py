"""CPU restatement of the learned block correction's network (test
infrastructure only: the tests compare the GPU kernels against it; nothing
in the product imports it).

Network (sayakaamr_gb300/csrc/mac_learned.h): per block of nb x nb cells,
3x3 convolutions with zero padding at the block edge, 3 -> 32 -> 32 -> 1
channels, ReLU after the first two.  Parameter vector (FP32):
w1[32][3][9], b1[32], w2[32][32][9], b2[32], w3[32][9], b3.
The output is projected onto the block-local part (its least-squares fit by
{1, x, y} over the block removed).  Loss of n blocks, for the correction
u = sa * P(y): mode 0, the residual u leaves under the block-local operator
A u = (K u) / (dv vf), (K u)_c = sum_f T_f (u_c - u_nb), u = 0 outside:
(1/n) * sum (feat0 - A u)^2; mode 1, the distance to the stored error
target e: (1/n) * sum (u - e)^2.  aux = [sa][dv vf][x-face T][y-face T][e].
No counterpart in the
reference library; pinned by finite differences in tests/test_nn_oracle.py.
"""
import numpy as np

C, CIN = 32, 3
OW1 = 0
OB1 = OW1 + C * CIN * 9
OW2 = OB1 + C
OB2 = OW2 + C * C * 9
OW3 = OB2 + C
OB3 = OW3 + C * 9
NPARAM = OB3 + 1


def unpack(w):
    w = np.asarray(w, dtype=np.float64)
    return (w[OW1:OB1].reshape(C, CIN, 3, 3), w[OB1:OW2], w[OW2:OB2].reshape(C, C, 3, 3), w[OB2:OW3],
            w[OW3:OB3].reshape(1, C, 3, 3), w[OB3:OB3 + 1])


def conv(x, k, b):
    """x [n][cin][H][W], k [cout][cin][3][3] (tap (dy, dx) at k[..., dy+1, dx+1]), zero padding"""
    n, cin, H, W = x.shape
    xp = np.zeros((n, cin, H + 2, W + 2))
    xp[:, :, 1:-1, 1:-1] = x
    out = np.zeros((n, k.shape[0], H, W)) + b[None, :, None, None]
    for dy in range(3):
        for dx in range(3):
            out += np.einsum("nchw,oc->nohw", xp[:, :, dy:dy + H, dx:dx + W], k[:, :, dy, dx])
    return out


def conv_grad(x, k, g):
    """gradients of conv(x, k, b) against k, b and x for the output gradient g"""
    n, cin, H, W = x.shape
    xp = np.zeros((n, cin, H + 2, W + 2))
    xp[:, :, 1:-1, 1:-1] = x
    gk = np.zeros_like(k)
    gxp = np.zeros_like(xp)
    for dy in range(3):
        for dx in range(3):
            gk[:, :, dy, dx] = np.einsum("nohw,nchw->oc", g, xp[:, :, dy:dy + H, dx:dx + W])
            gxp[:, :, dy:dy + H, dx:dx + W] += np.einsum("nohw,oc->nchw", g, k[:, :, dy, dx])
    return gk, g.sum(axis=(0, 2, 3)), gxp[:, :, 1:-1, 1:-1]


def local_part(v, nb):
    """v [n][nb*nb] minus its block-wise least-squares fit by {1, x, y}"""
    v = np.asarray(v, dtype=np.float64).reshape(-1, nb, nb)
    c = np.arange(nb) - 0.5 * (nb - 1)
    xi, yj = c[None, None, :], c[None, :, None]
    sxx = nb * nb * (nb * nb - 1) / 12.0
    a0 = v.mean(axis=(1, 2), keepdims=True)
    a1 = (v * xi).sum(axis=(1, 2), keepdims=True) / sxx
    a2 = (v * yj).sum(axis=(1, 2), keepdims=True) / sxx
    return (v - a0 - a1 * xi - a2 * yj).reshape(v.shape[0], nb * nb)


def forward(w, feat, nb, bf16=False, project=True):
    """y [n][nb*nb] for features [n][3][nb*nb]; bf16 rounds the hidden layer's
    operands to BF16 as the tensor-core inference does"""
    w1, b1, w2, b2, w3, b3 = unpack(w)
    x = np.asarray(feat, dtype=np.float64).reshape(-1, CIN, nb, nb)
    h1 = np.maximum(conv(x, w1, b1), 0.0)
    if bf16:
        h1, w2 = to_bf16(h1), to_bf16(w2)
    h2 = np.maximum(conv(h1, w2, b2), 0.0)
    y = conv(h2, w3, b3).reshape(x.shape[0], nb * nb)
    return local_part(y, nb) if project else y


def _K(u, tx, ty):
    """u [n][nb][nb] -> K u with u = 0 outside; tx [n][nb][nb+1], ty [n][nb+1][nb]"""
    up = np.pad(u, ((0, 0), (1, 1), (1, 1)))
    c = up[:, 1:-1, 1:-1]
    return (tx[:, :, :-1] * (c - up[:, 1:-1, :-2]) + tx[:, :, 1:] * (c - up[:, 1:-1, 2:]) +
            ty[:, :-1, :] * (c - up[:, :-2, 1:-1]) + ty[:, 1:, :] * (c - up[:, 2:, 1:-1]))


def split_aux(aux, nb):
    aux = np.asarray(aux, dtype=np.float64)
    n, nc, nf = aux.shape[0], nb * nb, (nb + 1) * nb
    sa = aux[:, :nc].reshape(n, nb, nb)
    dvvf = aux[:, nc:2 * nc].reshape(n, nb, nb)
    tx = aux[:, 2 * nc:2 * nc + nf].reshape(n, nb, nb + 1)
    ty = aux[:, 2 * nc + nf:2 * nc + 2 * nf].reshape(n, nb + 1, nb)
    e = aux[:, 2 * nc + 2 * nf:].reshape(n, nb, nb)
    return sa, dvvf, tx, ty, e


def loss_grad(w, feat, aux, nb, mode=1):
    w1, b1, w2, b2, w3, b3 = unpack(w)
    n = feat.shape[0]
    x = np.asarray(feat, dtype=np.float64).reshape(n, CIN, nb, nb)
    sa, dvvf, tx, ty, e = split_aux(aux, nb)
    a1 = conv(x, w1, b1)
    h1 = np.maximum(a1, 0.0)
    a2 = conv(h1, w2, b2)
    h2 = np.maximum(a2, 0.0)
    y = local_part(conv(h2, w3, b3)[:, 0].reshape(n, nb * nb), nb).reshape(n, nb, nb)
    u = sa * y
    if mode == 1:
        res = u - e
        loss = float(np.sum(res * res) / n)
        dldu = 2.0 * res / n
    else:
        inv = np.where(dvvf > 0, 1.0 / np.where(dvvf > 0, dvvf, 1.0), 0.0)
        res = x[:, 0] - _K(u, tx, ty) * inv
        loss = float(np.sum(res * res) / n)
        g = -2.0 * res / n
        dldu = _K(g * inv, tx, ty)
    gy = local_part((sa * dldu).reshape(n, nb * nb), nb).reshape(n, nb, nb)[:, None]
    g3, gb3, gh2 = conv_grad(h2, w3, gy)
    ga2 = gh2 * (a2 > 0)
    g2, gb2, gh1 = conv_grad(h1, w2, ga2)
    ga1 = gh1 * (a1 > 0)
    g1, gb1, _ = conv_grad(x, w1, ga1)
    grad = np.concatenate([g1.ravel(), gb1, g2.ravel(), gb2, g3.ravel(), gb3])
    return loss, grad


def random_aux(rng, n, nb):
    """plausible block-operator data for tests: positive face coefficients,
    dv*vf of a uniform block with a few solid cells"""
    nc, nf = nb * nb, (nb + 1) * nb
    sa = rng.uniform(0.1, 0.3, (n, nc))
    dvvf = np.where(rng.uniform(0, 1, (n, nc)) < 0.1, 0.0, 1.0)
    sa = sa * dvvf
    t = rng.uniform(0.5, 2.0, (n, 2 * nf))
    e = rng.normal(0.0, 0.1, (n, nc)) * dvvf
    return np.concatenate([sa, dvvf, t, e], axis=1).astype(np.float32)


def to_bf16(a):
    """round to the nearest BF16 (ties to even), returned as float64"""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def init(seed=0):
    rng = np.random.default_rng(seed)
    w = np.zeros(NPARAM)
    w[OW1:OB1] = rng.normal(0, np.sqrt(2 / (CIN * 9)), OB1 - OW1)
    w[OW2:OB2] = rng.normal(0, np.sqrt(2 / (C * 9)), OB2 - OW2)
    w[OW3:OB3] = rng.normal(0, 0.05, OB3 - OW3)
    w[OB1:OW2] = rng.normal(0, 0.05, C)
    w[OB2:OW3] = rng.normal(0, 0.05, C)
    return w.astype(np.float32)

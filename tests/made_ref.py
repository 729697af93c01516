"""numpy restatement of the learned proposal (MADE) for the tests: BF16
rounding of the weights, the masks and degrees, teacher-forced log q with the
magnetisation-sector forcing, and the mean NLL gradient by explicit backprop.
Layout (as the C API): W1t[N][H], b1[H], W2t[H][H], b2[H], W3t[H][N], b3[N]."""
import numpy as np


def bf16(a):
    """float32 -> nearest BF16 (ties to even), returned as float32."""
    b = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32)


def degrees(N, H):
    return 1 + (np.arange(H) * (N - 1)) // H


def masks(N, H):
    m = degrees(N, H)
    M1 = (m[None, :] >= np.arange(1, N + 1)[:, None])          # W1t[i][k]
    M2 = (m[None, :] >= m[:, None])                            # W2t[j][k]
    M3 = (np.arange(1, N + 1)[None, :] > m[:, None])           # W3t[k][i]
    return M1, M2, M3


def unpack(w, N, H):
    o = 0
    W1 = w[o:o + N * H].reshape(N, H); o += N * H
    b1 = w[o:o + H]; o += H
    W2 = w[o:o + H * H].reshape(H, H); o += H * H
    b2 = w[o:o + H]; o += H
    W3 = w[o:o + H * N].reshape(H, N); o += H * N
    b3 = w[o:o + N]
    return W1, b1, W2, b2, W3, b3


def num_params(N, H):
    return N * H + H + H * H + H + H * N + N


def mask_vector(N, H):
    M1, M2, M3 = masks(N, H)
    return np.concatenate([M1.ravel(), np.ones(H), M2.ravel(), np.ones(H), M3.ravel(), np.ones(N)]).astype(bool)


def free_sites(x, n_ones):
    """x: [B][N] 0/1 (1 = down spin); True where site i is not forced by the sector."""
    B, N = x.shape
    if n_ones < 0:
        return np.ones_like(x, dtype=bool)
    before = np.concatenate([np.zeros((B, 1), int), np.cumsum(x, axis=1)[:, :-1]], axis=1)
    need = n_ones - before
    rem = N - np.arange(N)[None, :]
    return (need > 0) & (need < rem)


def forward(w, x, N, H):
    W1, b1, W2, b2, W3, b3 = [bf16(a).astype(np.float64) for a in unpack(np.where(mask_vector(N, H), w, 0), N, H)]
    a1 = x @ W1 + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2 + b2
    h2 = np.maximum(a2, 0)
    logit = h2 @ W3 + b3
    return a1, h1, a2, h2, logit, (W1, W2, W3)


def log_sigmoid(l):
    return -np.logaddexp(0.0, -l)


def logq(w, x, N, H, n_ones):
    *_, logit, _ = forward(w, x, N, H)
    lp = np.where(x == 1, log_sigmoid(logit), log_sigmoid(-logit))
    return np.sum(np.where(free_sites(x, n_ones), lp, 0.0), axis=1)


def nll_grad(w, x, N, H, n_ones):
    """Mean NLL over the batch and its gradient in the layout (masked)."""
    a1, h1, a2, h2, logit, (W1, W2, W3) = forward(w, x, N, H)
    free = free_sites(x, n_ones)
    lp = np.where(x == 1, log_sigmoid(logit), log_sigmoid(-logit))
    nll = -np.sum(np.where(free, lp, 0.0)) / x.shape[0]
    dl = np.where(free, 1.0 / (1.0 + np.exp(-logit)) - x, 0.0) / x.shape[0]
    gW3 = h2.T @ dl
    gb3 = dl.sum(0)
    dh2 = dl @ W3.T
    da2 = dh2 * (a2 > 0)
    gW2 = h1.T @ da2
    gb2 = da2.sum(0)
    dh1 = da2 @ W2.T
    da1 = dh1 * (a1 > 0)
    gW1 = x.T @ da1
    gb1 = da1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return nll, np.where(mask_vector(N, H), g, 0.0)


def bits_of(spins):
    """+-1 spins -> 0/1 with 1 = down."""
    return (np.asarray(spins) < 0).astype(np.int64)

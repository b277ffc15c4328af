"""NumPy restatement of the radiance-cache network for the tests: the same
hash-grid encoding, BF16 rounding of every layer input and weight, float64
accumulation, and the backward pass of the relative L2 loss."""

import numpy as np

LEVELS, TABLE, IN, HID, OUT = 16, 1 << 19, 48, 64, 16
DIMS = [(64, 48), (64, 64), (64, 64), (64, 64), (64, 64), (16, 64)]


def bf16(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint32) << 16
    return u.view(np.float32).astype(np.float64)


def level_res():
    b = np.exp((np.log(np.float32(2048)) - np.log(np.float32(16))) / np.float32(LEVELS - 1))
    return np.floor(np.float32(16) * np.power(np.float32(b), np.arange(LEVELS, dtype=np.float32)))


def grid_index(x, y, z, side):
    if side ** 3 <= TABLE:
        return x + side * (y + side * z)
    h = (x.astype(np.uint64) ^ (y.astype(np.uint64) * 2654435761) ^ (z.astype(np.uint64) * 805459861))
    return (h & np.uint64(TABLE - 1)).astype(np.int64)


def batch_grid_index(x, y, z, side, cell):
    """A batch cache's vertex: coordinates offset by side x the cell, hashed."""
    xs = (x + side * cell[:, 0]).astype(np.uint64)
    ys = (y + side * cell[:, 1]).astype(np.uint64)
    zs = (z + side * cell[:, 2]).astype(np.uint64)
    h = xs ^ ((ys * np.uint64(2654435761)) & np.uint64(0xFFFFFFFF)) ^ \
        ((zs * np.uint64(805459861)) & np.uint64(0xFFFFFFFF))
    return (h & np.uint64(TABLE - 1)).astype(np.int64)


def corners(q, lo, hi):
    """Per level: (indices [n, 8], weights [n, 8]).  lo None: positions in
    batch-cell coordinates (x in [0, 1]^3 plus twice an integer cell)."""
    pos = q[:, :3].astype(np.float32)
    if lo is None:
        cell = np.clip(np.floor(pos * np.float32(0.5)), 0, 15).astype(np.float32)
        p = np.clip(pos - np.float32(2) * cell, 0, 1).astype(np.float32)
        cell = cell.astype(np.int64)
    else:
        lo = np.asarray(lo, np.float32)
        inv = (np.float32(1) / np.maximum(np.asarray(hi, np.float32) - lo, np.float32(1e-6)))
        p = np.clip((pos - lo) * inv, 0, 1).astype(np.float32)
        cell = None
    out = []
    for res in level_res():
        side = int(res) + 1
        x = p * np.float32(res)
        c0 = np.minimum(np.floor(x), np.float32(res - 1))
        fr = (x - c0).astype(np.float64)
        c0 = c0.astype(np.int64)
        idx, w = [], []
        for c in range(8):
            o = np.array([c & 1, (c >> 1) & 1, (c >> 2) & 1])
            g = c0 + o
            if cell is None:
                idx.append(grid_index(g[:, 0], g[:, 1], g[:, 2], side))
            else:
                idx.append(batch_grid_index(g[:, 0], g[:, 1], g[:, 2], side, cell))
            w.append(np.prod(np.where(o == 1, fr, 1 - fr), axis=1))
        out.append((np.stack(idx, 1), np.stack(w, 1)))
    return out


def encode(q, table, lo, hi):
    cs = corners(q, lo, hi)
    feats = []
    for l, (idx, w) in enumerate(cs):
        e = table[l][idx].astype(np.float64)  # [n, 8, 2]
        feats.append((w[:, :, None] * e).sum(1))
    x = np.zeros((q.shape[0], IN))
    x[:, :32] = np.concatenate(feats, 1)
    x[:, 32:41] = q[:, 3:12]
    return x, cs


def split(weights):
    out, off = [], 0
    for o, i in DIMS:
        out.append(np.asarray(weights[off:off + o * i], np.float64).reshape(o, i))
        off += o * i
    return out


def forward(q, weights, table, lo, hi):
    x, cs = encode(q, table, lo, hi)
    acts = [bf16(x)]
    ws = [bf16(w) for w in split(weights)]
    h = acts[0]
    for l, w in enumerate(ws):
        y = h @ w.T
        if l + 1 < len(ws):
            h = bf16(np.maximum(y, 0))
            acts.append(h)
    return y[:, :3], acts, ws, cs


def gradients(records, weights, table, lo, hi):
    """Mean relative L2 loss and d/d(weights), d/d(table) as the kernels
    compute them (dLoss/dY rounded to BF16 between layers)."""
    q = records[:, :12]
    t = records[:, 12:15].astype(np.float64)
    n = q.shape[0]
    pred, acts, ws, cs = forward(q, weights, table, lo, hi)
    den = pred * pred + 0.01
    loss = ((pred - t) ** 2 / den).sum() / n
    dy = np.zeros((n, OUT))
    dy[:, :3] = 2 * (pred - t) / den / n
    dy = bf16(dy)
    gw = [None] * len(ws)
    for l in range(len(ws) - 1, -1, -1):
        gw[l] = dy.T @ acts[l]
        dx = dy @ ws[l]
        if l > 0:
            dy = bf16(np.where(acts[l] > 0, dx, 0))
        else:
            dfeat = dx[:, :32]
    gw[-1][3:] = 0
    gt = np.zeros((LEVELS, TABLE, 2))
    for l, (idx, w) in enumerate(cs):
        for c in range(8):
            np.add.at(gt[l], idx[:, c], w[:, c:c + 1] * dfeat[:, 2 * l:2 * l + 2])
    return loss, np.concatenate([g.ravel() for g in gw]), gt

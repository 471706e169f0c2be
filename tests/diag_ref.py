"""numpy restatement of the microstructure diagnostics (test reference):
same definitions as the device kernels -- level-set area/perimeter/box,
dominant-order-parameter labels, 4-neighbour connected components through
periodic wraps (union-find), boundary edges per label pair."""
import numpy as np


def interface(f, level, dx, dy, bc):
    a = f >= level
    if bc == 0:
        ex = np.sum(a != np.roll(a, -1, axis=1))
        ey = np.sum(a != np.roll(a, -1, axis=0))
    else:
        ex = np.sum(a[:, :-1] != a[:, 1:])
        ey = np.sum(a[:-1, :] != a[1:, :])
    ys, xs = np.nonzero(a)
    box = (xs.min(), xs.max(), ys.min(), ys.max()) if len(xs) else (-1, -1, -1, -1)
    return int(a.sum()), float(a.sum()) * dx * dy, ex * dy + ey * dx, box


def labels(etas, thr, conc=None, clevel=0.5):
    lab = np.argmax(etas, axis=0)
    mx = np.max(etas, axis=0)
    lab = np.where(mx >= thr, lab, -1)
    if conc is not None:
        lab = np.where(conc >= clevel, lab, -1)
    return lab


def components(lab, bc):
    ny, nx = lab.shape
    parent = np.arange(ny * nx)

    def find(i):
        while parent[i] != i:
            parent[i] = parent[parent[i]]
            i = parent[i]
        return i

    def union(a, b):
        ra, rb = find(a), find(b)
        if ra != rb:
            parent[max(ra, rb)] = min(ra, rb)

    for y in range(ny):
        for x in range(nx):
            l = lab[y, x]
            if l < 0:
                continue
            for (xx, yy) in ((x + 1, y), (x, y + 1)):
                if bc == 0:
                    xx %= nx
                    yy %= ny
                elif xx >= nx or yy >= ny:
                    continue
                if lab[yy, xx] == l:
                    union(y * nx + x, yy * nx + xx)
    roots = {find(i) for i in range(ny * nx) if lab.flat[i] >= 0}
    return len(roots), int((lab >= 0).sum())


def boundaries(lab, q, dx, dy, bc):
    out = np.zeros((q, q))
    pairs = [((lambda a: np.roll(a, -1, axis=1)) if bc == 0 else None, dy, 1),
             ((lambda a: np.roll(a, -1, axis=0)) if bc == 0 else None, dx, 0)]
    for shift, w, axis in pairs:
        if bc == 0:
            a, b = lab, shift(lab)
        else:
            a, b = (lab[:, :-1], lab[:, 1:]) if axis == 1 else (lab[:-1, :], lab[1:, :])
        m = (a >= 0) & (b >= 0) & (a != b)
        for u, v in zip(a[m], b[m]):
            out[u, v] += w
            out[v, u] += w
    return out

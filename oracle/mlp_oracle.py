"""NumPy oracle of the acoustic-cycle surrogate (test infrastructure only).

Only tests/ import this module, as the checker of the GPU surrogate.  The
surrogate has no counterpart in the reference; what it approximates is one
call of sound() (nompi/mod_moloch.F90:483-851), and the parts restated here
are the ones the GPU computes:

* features(): the 45*kz inputs of a column -- u, v, w (levels 2..kz+1), pai
  and tetav of the column and its 8 periodic neighbours, feature index
  (f*kz + k)*9 + nb with nb = (di+1)*3 + (dj+1);
* forward() / backward(): the MLP 45kz -> 256 -> 256 -> 256 -> 5kz with SiLU,
  mean-squared-error loss and its gradients, with the GPU's BF16 roundings
  (operands and stored activations rounded to nearest-even BF16, products
  accumulated in high precision) so that the tensor-core results can be
  compared element by element;
* apply(): committing an accepted cycle -- state plus denormalised
  increments, and the generalised vertical velocity s of Equation 10
  (nompi/mod_moloch.F90:557-570 and :843-849) evaluated with the new w and
  the winds at the start of the last substep, taken as the pre-cycle winds
  plus (nsound-1)/nsound of the predicted increment.
"""
import numpy as np

FIELDS = ("u", "v", "w", "pai", "tetav")


def bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    a = np.ascontiguousarray(np.asarray(x, np.float32)).view(np.uint32)
    r = ((a >> 16) & np.uint32(1)) + np.uint32(0x7FFF)
    return ((a + r) & np.uint32(0xFFFF0000)).view(np.float32)


def silu(z):
    return z / (1.0 + np.exp(-z))


def features(st):
    """Raw features [ncol][45*kz] from a dict of (kz, ni, nj) arrays; for w
    the (kz+1, ni, nj) array."""
    u = st["u"]
    kz, ni, nj = u.shape
    flds = (st["u"], st["v"], st["w"][1:kz + 1], st["pai"], st["tetav"])
    out = np.empty((ni * nj, 5, kz, 9), np.float64)
    for di in (-1, 0, 1):
        for dj in (-1, 0, 1):
            nb = (di + 1) * 3 + (dj + 1)
            for f, a in enumerate(flds):
                sh = np.roll(np.roll(a, -di, axis=1), -dj, axis=2)  # value at (i+di, j+dj)
                out[:, f, :, nb] = sh.reshape(kz, ni * nj).T
    return out.reshape(ni * nj, 45 * kz)


def normalise(X, xmean, xstd, kin):
    """Normalised features padded with zeros to kin columns."""
    n, nin = X.shape
    m = np.asarray(xmean, np.float64).ravel()
    s = np.asarray(xstd, np.float64).ravel()
    idx = np.arange(nin) // 9  # statistic of field plane f * kz + k
    out = np.zeros((n, kin))
    out[:, :nin] = (X - m[idx]) / s[idx]
    return out


def forward(params, X, rnd=True):
    """Returns (Y, Z, H): Z the three pre-activations, H[0] the (rounded)
    input and H[1..3] the stored activations."""
    q = bf16 if rnd else (lambda a: a)
    h = np.asarray(q(X), np.float64)
    Z, H = [], [h]
    for l in range(3):
        W, b = params[l]
        z = h @ np.asarray(q(W), np.float64).T + b
        Z.append(z)
        h = np.asarray(q(silu(z)), np.float64)
        H.append(h)
    W, b = params[3]
    return h @ np.asarray(q(W), np.float64).T + b, Z, H


def backward(params, X, T, m, rnd=True):
    """Summed squared error over the first m outputs and the gradients
    [(dW, db)] * 4 of the mean squared error."""
    q = bf16 if rnd else (lambda a: a)
    Y, Z, H = forward(params, X, rnd)
    n = X.shape[0]
    e = np.zeros_like(Y)
    e[:, :m] = Y[:, :m] - T[:, :m]
    loss = float(np.sum(e * e))
    d = np.asarray(q(2.0 * e / (n * m)), np.float64)
    grads = [None] * 4
    grads[3] = (d.T @ H[3], d.sum(axis=0))
    dH = d @ np.asarray(q(params[3][0]), np.float64)
    for l in (2, 1, 0):
        z = Z[l]
        sg = 1.0 / (1.0 + np.exp(-z))
        dz = np.asarray(q(dH * (sg * (1.0 + z * (1.0 - sg)))), np.float64)
        grads[l] = (dz.T @ H[l], dz.sum(axis=0))
        if l > 0:
            dH = dz @ np.asarray(q(params[l][0]), np.float64)
    return loss, grads


def apply(st, inc, nsound, hx, hy, gzitak, fmzf):
    """Post-cycle state from the pre-cycle state st (dict as in features(),
    plus nothing else) and increments inc [5][kz][ni][nj].  hx, hy (ni, nj)
    interior; gzitak (kz+1,) the metric factor at the full levels; fmzf
    (kz+1, ni, nj).  Returns a dict with u, v, w, pai, tetav and s."""
    kz = st["u"].shape[0]
    out = {f: np.array(st[f], np.float64) for f in FIELDS}
    out["u"] += inc[0]
    out["v"] += inc[1]
    out["w"][1:kz + 1] += inc[2]
    out["pai"] += inc[3]
    out["tetav"] += inc[4]
    fr = (nsound - 1) / nsound
    ul = st["u"] + fr * inc[0]
    vl = st["v"] + fr * inc[1]
    ue = np.roll(ul, -1, axis=2)
    vn = np.roll(vl, -1, axis=1)
    hxe = np.roll(hx, -1, axis=1)
    hyn = np.roll(hy, -1, axis=0)
    s = np.zeros((kz + 1,) + hx.shape)
    for k in range(1, kz):
        zuh = (ul[k] + ul[k - 1]) * hx + (ue[k] + ue[k - 1]) * hxe
        zvh = (vl[k] + vl[k - 1]) * hy + (vn[k] + vn[k - 1]) * hyn
        s[k] = (out["w"][k] - 0.25 * (zuh + zvh) * gzitak[k]) * fmzf[k]
    out["s"] = s
    return out


def gzita(zita, ztop, a0):
    """Vertical metric decay function, nompi/mod_zita.F90:109-120."""
    r = np.asarray(zita, np.float64) / ztop
    return (((0.0 - a0) * r - (3.0 - 2.0 * a0) * r * r) + (2.0 - a0) * r ** 3) + 1.0

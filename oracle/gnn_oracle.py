"""CPU ORACLE for the learned chain preconditioner -- test infrastructure only.

numpy restatement of the coefficient network, its probe loss and gradient,
used by tests/ to check the device's BF16 forward / backward kernels.  This
component has no counterpart in the reference (maplab's Ceres path uses a
SCHUR_JACOBI preconditioner); its definition is:

* reduced camera system S (15x15 keyframe blocks): diag[k], pose-pose
  upper[b] (6x6, rows i, columns j for upper_ij[b] = (i, j), i < j) and
  inertial[e] (15x15, rows from, columns to);
* chain order perm (position -> keyframe), link_edge[p] / link_blk[p]: the
  inertial edge and oriented pose block coupling position p to p - 1;
* chain matrix T(coef): T_pp = S_kk + alpha_p diag(comp_p) on the active pose
  rows, comp_p = off-chain |S| row sums of the pose rows; T_{p,p-1} =
  gamma_ine,p E^T + gamma_vis,p P (E the (kf(p-1), kf(p)) inertial block, P
  the (kf(p), kf(p-1)) pose block);
* network: couplings c_kj = |S_kj|_F / sqrt(|S_kk|_F |S_jj|_F); features;
  3 layers m = sum c h / sum c, z = W1 h + W2 m + b, h' = relu(z); head
  o = Wh [h_k; h_k'] + bh, gamma = sig(o0), sig(o1), alpha = 0.1 sig(o2);
* loss L = mean over probes of |T^-1 S w - w|^2 / (15 N_kf); gradient by the
  adjoint lambda = T^-1 (2 e / (P n)): dL/dT = -lambda y^T.

With bf16=True the device's rounding points are reproduced (inputs, layer
outputs, aggregated inputs and pre-activation gradients rounded to BF16,
weights used as BF16); with bf16=False everything is FP64 (finite-difference
checks of the restatement itself).
"""
import numpy as np

HID, IN, LAYERS, OUT, ALPHA_MAX = 64, 32, 3, 3, 0.1


def layout():
    off, L = 0, {}
    for l in range(LAYERS):
        k = IN if l == 0 else HID
        L[f"w1_{l}"] = (off, (HID, k)); off += HID * k
        L[f"w2_{l}"] = (off, (HID, k)); off += HID * k
        L[f"b_{l}"] = (off, (HID,)); off += HID
    L["wh"] = (off, (OUT, 2 * HID)); off += OUT * 2 * HID
    L["bh"] = (off, (OUT,)); off += OUT
    return L, off


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, use_bf16):
    L, _ = layout()
    out = {}
    for name, (o, shp) in L.items():
        v = np.asarray(params[o:o + int(np.prod(shp))], dtype=np.float64).reshape(shp)
        if use_bf16 and not name.startswith("b"):
            v = bf16(v)
        out[name] = v
    return out


def sig(x):
    return 1.0 / (1.0 + np.exp(-x))


class ChainProblem:
    """The reduced system and chain structure in the device's export format."""

    def __init__(self, sysd, perm, link_edge, link_blk, mask=None):
        self.D = sysd["diag"]
        self.U = sysd["upper"]
        self.ij = sysd["upper_ij"]
        self.E = sysd["inertial"]
        self.ef = sysd["edge_from"]
        self.et = sysd["edge_to"]
        self.perm, self.le, self.lb = perm, link_edge, link_blk
        self.n = self.D.shape[0]
        self.npu = self.U.shape[0]
        if mask is None:  # fixed dims are identity rows with no coupling
            mask = np.ones((self.n, 15), dtype=bool)
            for k in range(self.n):
                for d in range(15):
                    row = self.D[k, d].copy(); row[d] = 0.0
                    if self.D[k, d, d] == 1.0 and not row.any():
                        mask[k, d] = False
        self.mask = mask
        # neighbour lists: pose blocks (oriented) then inertial edges
        self.nbr = [[] for _ in range(self.n)]
        for b, (i, j) in enumerate(self.ij):
            self.nbr[i].append((j, self.U[b]))
            self.nbr[j].append((i, self.U[b].T))
        for e, (f, t) in enumerate(zip(self.ef, self.et)):
            self.nbr[f].append((t, self.E[e]))
            self.nbr[t].append((f, self.E[e].T))
        self.pos = np.empty(self.n, dtype=np.int64)
        self.pos[perm] = np.arange(self.n)

    def oriented_pose(self, lb):
        return self.U[lb] if lb < self.npu else self.U[lb - self.npu].T

    def linked(self, p):
        return p > 0 and (self.le[p] >= 0 or self.lb[p] >= 0)

    def dense_S(self):
        n = self.n
        S = np.zeros((15 * n, 15 * n))
        for k in range(n):
            S[15 * k:15 * k + 15, 15 * k:15 * k + 15] = self.D[k]
        for b, (i, j) in enumerate(self.ij):
            S[15 * i:15 * i + 6, 15 * j:15 * j + 6] += self.U[b]
            S[15 * j:15 * j + 6, 15 * i:15 * i + 6] += self.U[b].T
        for e, (f, t) in enumerate(zip(self.ef, self.et)):
            S[15 * f:15 * f + 15, 15 * t:15 * t + 15] += self.E[e]
            S[15 * t:15 * t + 15, 15 * f:15 * f + 15] += self.E[e].T
        return S

    def comp(self):
        """Off-chain |S| row sums of the pose rows per chain position."""
        c = np.zeros((self.n, 6))
        for p in range(self.n):
            k = self.perm[p]
            excl = set()
            if self.linked(p):
                excl.add(self.perm[p - 1])
            if p + 1 < self.n and self.linked(p + 1):
                excl.add(self.perm[p + 1])
            for b, (i, j) in enumerate(self.ij):
                if i == k and j not in excl:
                    c[p] += np.abs(self.U[b]).sum(axis=1)
                elif j == k and i not in excl:
                    c[p] += np.abs(self.U[b].T).sum(axis=1)
        return c

    def link_blocks(self, p):
        """(E^T or 0, P or 0) of T(p, p-1)."""
        Ep = self.E[self.le[p]].T if self.le[p] >= 0 else np.zeros((15, 15))
        Pp = np.zeros((15, 15))
        if self.lb[p] >= 0:
            Pp[:6, :6] = self.oriented_pose(self.lb[p])
        return Ep, Pp

    def dense_T(self, coef):
        n = self.n
        T = np.zeros((15 * n, 15 * n))
        comp = self.comp()
        for p in range(n):
            k = self.perm[p]
            blk = self.D[k].copy()
            for r in range(6):
                if self.mask[k, r]:
                    blk[r, r] += coef[p, 2] * comp[p, r]
            T[15 * k:15 * k + 15, 15 * k:15 * k + 15] = blk
            if p > 0:
                kq = self.perm[p - 1]
                Ep, Pp = self.link_blocks(p)
                B = coef[p, 0] * Ep + coef[p, 1] * Pp
                T[15 * k:15 * k + 15, 15 * kq:15 * kq + 15] = B
                T[15 * kq:15 * kq + 15, 15 * k:15 * k + 15] = B.T
        return T, comp


def features(cp, use_bf16):
    n = cp.n
    nrm = np.array([max(np.linalg.norm(cp.D[k]), 1e-30) for k in range(n)])
    wgt = [[np.linalg.norm(B) / np.sqrt(nrm[k] * nrm[j]) for j, B in cp.nbr[k]] for k in range(n)]
    deg = np.array([sum(w) for w in wgt])
    x = np.zeros((n, IN))
    for p in range(n):
        k = cp.perm[p]
        kp = cp.perm[p - 1] if cp.linked(p) else -1
        kn = cp.perm[p + 1] if (p + 1 < n and cp.linked(p + 1)) else -1
        cpv = sum(w for (j, _), w in zip(cp.nbr[k], wgt[k]) if j == kp)
        cnv = sum(w for (j, _), w in zip(cp.nbr[k], wgt[k]) if j == kn)
        x[k, :15] = np.log10(np.maximum(np.diag(cp.D[k]), 1e-12)) * 0.1
        x[k, 15] = np.log2(1.0 + len(cp.nbr[k])) * 0.125
        x[k, 16] = deg[k] - cpv - cnv
        x[k, 17] = cpv
        x[k, 18] = cnv
        x[k, 19] = 1.0
    if use_bf16:
        x = bf16(x)
    return x, wgt, deg


def forward(cp, params, use_bf16=True):
    P = unpack(params, use_bf16)
    rnd = bf16 if use_bf16 else (lambda v: v)
    x, wgt, deg = features(cp, use_bf16)
    n = cp.n
    hs, ms, zs = [x], [], []
    h = x
    for l in range(LAYERS):
        m = np.zeros_like(h)
        for k in range(n):
            for (j, _), c in zip(cp.nbr[k], wgt[k]):
                m[k] += c * h[j]
            if deg[k] > 0:
                m[k] /= deg[k]
        m = rnd(m)
        z = h @ P[f"w1_{l}"].T + m @ P[f"w2_{l}"].T + P[f"b_{l}"]
        h = rnd(np.maximum(z, 0.0))
        ms.append(m); zs.append(z); hs.append(h)
    o = np.zeros((n, OUT))
    g_in = np.zeros((n, 2 * HID))
    for p in range(n):
        k = cp.perm[p]
        g = np.zeros(2 * HID)
        g[:HID] = h[k]
        if cp.linked(p):
            g[HID:] = h[cp.perm[p - 1]]
        g_in[p] = g
        o[p] = P["wh"] @ g + P["bh"]
    coef = np.stack([sig(o[:, 0]), sig(o[:, 1]), ALPHA_MAX * sig(o[:, 2])], axis=1)
    return dict(P=P, x=x, wgt=wgt, deg=deg, hs=hs, ms=ms, zs=zs, o=o, g_in=g_in, coef=coef)


def loss_and_grad(cp, params, probes, use_bf16=True):
    """Loss and gradient w.r.t. the flat parameter vector (and d loss / d coef)."""
    f = forward(cp, params, use_bf16)
    P, coef = f["P"], f["coef"]
    rnd = bf16 if use_bf16 else (lambda v: v)
    S = cp.dense_S()
    T, comp = cp.dense_T(coef)
    n15 = 15 * cp.n
    scale = 1.0 / (len(probes) * n15)
    loss = 0.0
    dcoef = np.zeros((cp.n, 3))
    for w in probes:
        y = np.linalg.solve(T, S @ w)
        e = y - w
        loss += scale * float(e @ e)
        lam = np.linalg.solve(T, 2.0 * scale * e)
        Y, Lm = y.reshape(cp.n, 15), lam.reshape(cp.n, 15)
        for p in range(cp.n):
            k = cp.perm[p]
            dcoef[p, 2] -= sum(Lm[k, r] * comp[p, r] * Y[k, r] for r in range(6) if cp.mask[k, r])
            if p > 0:
                kq = cp.perm[p - 1]
                Ep, Pp = cp.link_blocks(p)
                dcoef[p, 0] -= Lm[k] @ Ep @ Y[kq] + Lm[kq] @ Ep.T @ Y[k]
                dcoef[p, 1] -= Lm[k] @ Pp @ Y[kq] + Lm[kq] @ Pp.T @ Y[k]
    # head
    L, total = layout()
    grad = np.zeros(total)

    def put(name, v):
        o, shp = L[name]
        grad[o:o + v.size] += v.ravel()

    o = f["o"]
    do = np.zeros_like(o)
    for q in range(3):
        sgm = sig(o[:, q])
        do[:, q] = dcoef[:, q] * sgm * (1 - sgm) * (ALPHA_MAX if q == 2 else 1.0)
    put("wh", do.T @ f["g_in"])
    put("bh", do.sum(axis=0))
    dh = np.zeros((cp.n, HID))
    dg = do @ P["wh"]
    for p in range(cp.n):
        k = cp.perm[p]
        dh[k] += dg[p, :HID]
        if cp.linked(p):
            dh[cp.perm[p - 1]] += dg[p, HID:]
    for l in range(LAYERS - 1, -1, -1):
        dz = rnd(dh * (f["zs"][l] > 0))
        put(f"b_{l}", dz.sum(axis=0))
        put(f"w1_{l}", dz.T @ f["hs"][l])
        put(f"w2_{l}", dz.T @ f["ms"][l])
        if l == 0:
            break
        dh = dz @ P[f"w1_{l}"]
        dm = dz @ P[f"w2_{l}"]
        for j in range(cp.n):
            for (i, _), c in zip(cp.nbr[j], f["wgt"][j]):
                if f["deg"][i] > 0:
                    dh[j] += c / f["deg"][i] * dm[i]
    return loss, grad, dcoef, coef


def random_chain_problem(n=12, seed=0):
    """Small well-conditioned system in the export format (tests of the
    restatement itself): one chain 0..n-1 with inertial and pose links plus a
    few off-chain pose blocks."""
    rng = np.random.default_rng(seed)
    D = np.zeros((n, 15, 15))
    for k in range(n):
        X = rng.normal(size=(15, 15)) * 0.3
        D[k] = X @ X.T + 6.0 * np.eye(15)
    pairs = [(k, k + 1) for k in range(n - 1)] + [(k, k + 3) for k in range(0, n - 3, 2)]
    U = np.stack([rng.normal(size=(6, 6)) * 0.4 for _ in pairs])
    E = np.stack([rng.normal(size=(15, 15)) * 0.3 for _ in range(n - 1)])
    sysd = dict(diag=D, upper=U, upper_ij=np.array(pairs, dtype=np.int32), inertial=E,
                edge_from=np.arange(n - 1, dtype=np.int32), edge_to=np.arange(1, n, dtype=np.int32))
    npu = len(pairs)
    perm = np.arange(n, dtype=np.int32)
    le = np.array([-1] + list(range(n - 1)), dtype=np.int32)
    lb = np.array([-1] + [npu + b for b in range(n - 1)], dtype=np.int32)  # (k, k-1) = transpose of upper (k-1, k)
    return ChainProblem(sysd, perm, le, lb)

"""FP64 CPU restatement of the learned candidate proposal (test infrastructure only).

Same parameter layout, hash-grid encoding, MLP and weighted softmax cross-entropy as
smallproject_gb300/csrc/proposal.cu, evaluated in float64 with an explicit backward
pass. Used to check the GPU's FP32 gradients and its BF16 inference probabilities.
"""
import numpy as np

IN, FEAT, LEVELS = 32, 8, 2


def layout(H, K, table_log2=16):
    T = 1 << table_log2
    o = {}
    off = 0
    for name, size in (("enc", LEVELS * T * FEAT), ("W1", H * IN), ("b1", H), ("W2", H * H), ("b2", H),
                       ("W3", H * H), ("b3", H), ("W4", K * H), ("b4", K)):
        o[name] = (off, size)
        off += size
    o["total"] = off
    o["T"] = T
    return o


def _hash(x, y, z, mask):
    x = x.astype(np.uint64)
    y = y.astype(np.uint64)
    z = z.astype(np.uint64)
    h = (x ^ ((y * np.uint64(2654435761)) & np.uint64(0xFFFFFFFF)) ^ ((z * np.uint64(805459861)) & np.uint64(0xFFFFFFFF)))
    return (h & np.uint64(mask)).astype(np.int64)


def corners(pos, res0, res1, T):
    """per level: (indices [B, 8] into the level-major table, weights [B, 8])"""
    out = []
    for l, R in enumerate((res0, res1)):
        s = np.float32(R) * np.float32(1.0 / 1024.0)
        u = np.clip(pos.astype(np.float32) * s, np.float32(0), np.float32(R)).astype(np.float32)
        i = np.minimum(u.astype(np.int64), R - 1)
        f = (u - i.astype(np.float32)).astype(np.float64)
        idx = np.zeros((pos.shape[0], 8), np.int64)
        w = np.zeros((pos.shape[0], 8), np.float64)
        for q in range(8):
            o = np.array([q & 1, (q >> 1) & 1, q >> 2])
            c = i + o
            idx[:, q] = l * T + _hash(c[:, 0], c[:, 1], c[:, 2], T - 1)
            w[:, q] = np.prod(np.where(o == 1, f, 1.0 - f), axis=1)
        out.append((idx, w))
    return out


def unpack(params, H, K, table_log2):
    L = layout(H, K, table_log2)
    p = np.asarray(params, np.float64)
    g = lambda n: p[L[n][0]:L[n][0] + L[n][1]]
    return L, {"enc": g("enc").reshape(LEVELS * L["T"], FEAT), "W1": g("W1").reshape(H, IN), "b1": g("b1"),
               "W2": g("W2").reshape(H, H), "b2": g("b2"), "W3": g("W3").reshape(H, H), "b3": g("b3"),
               "W4": g("W4").reshape(K, H), "b4": g("b4")}


def inputs(P, samples, res0, res1, T):
    s = np.asarray(samples, np.float32).reshape(-1, 4)
    pos = s[:, :3]
    code = s[:, 3].view(np.uint32)
    cs = corners(pos, res0, res1, T)
    X = np.zeros((s.shape[0], IN))
    for l, (idx, w) in enumerate(cs):
        X[:, l * FEAT:(l + 1) * FEAT] = np.einsum("bq,bqf->bf", w, P["enc"][idx])
    for k in range(6):
        X[:, 16 + k] = (code == k).astype(np.float64)
    return X, cs


def forward(params, samples, H, K, table_log2=16, res0=32, res1=128):
    L, P = unpack(params, H, K, table_log2)
    X, cs = inputs(P, samples, res0, res1, L["T"])
    H1 = np.maximum(X @ P["W1"].T + P["b1"], 0)
    H2 = np.maximum(H1 @ P["W2"].T + P["b2"], 0)
    H3 = np.maximum(H2 @ P["W3"].T + P["b3"], 0)
    Z = H3 @ P["W4"].T + P["b4"]
    return (L, P, X, cs, H1, H2, H3, Z)


def bf16(x):
    """Round to the nearest BF16 value, ties to even (cvt.rn.bf16.f32), as float64."""
    x = np.asarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def softmax(Z):
    e = np.exp(Z - Z.max(axis=1, keepdims=True))
    return e / e.sum(axis=1, keepdims=True)


def loss_and_grad(params, samples, target, weight, H, K, table_log2=16, res0=32, res1=128, bf16_operands=False):
    """Weighted softmax cross-entropy and its gradient in FP64. bf16_operands=True rounds
    every tensor-core operand to BF16 where the tensor-core training step rounds it (the
    network input, the four weight matrices, the three hidden activations, dZ, dH3, dH2,
    dH1), so the result is the gradient of the BF16 network that step differentiates."""
    L, P, X, cs, H1, H2, H3, Z = forward(params, samples, H, K, table_log2, res0, res1)
    r = bf16 if bf16_operands else (lambda a: a)
    if bf16_operands:
        X = r(X)
        P = dict(P)
        for n in ("W1", "W2", "W3", "W4"):
            P[n] = r(P[n])
        H1 = r(np.maximum(X @ P["W1"].T + P["b1"], 0))
        H2 = r(np.maximum(H1 @ P["W2"].T + P["b2"], 0))
        H3 = r(np.maximum(H2 @ P["W3"].T + P["b3"], 0))
        Z = H3 @ P["W4"].T + P["b4"]
    w = np.asarray(weight, np.float64)
    t = np.asarray(target, np.int64)
    ws = w.sum()
    wn = w / ws if ws > 0 else w * 0
    p = softmax(Z)
    B = Z.shape[0]
    loss = float(np.sum(wn * -np.log(p[np.arange(B), t])))
    dZ = p.copy()
    dZ[np.arange(B), t] -= 1.0
    dZ *= wn[:, None]
    g = {}
    dZ = r(dZ)
    g["W4"] = dZ.T @ H3
    g["b4"] = dZ.sum(0)
    dH3 = r((dZ @ P["W4"]) * (H3 > 0))
    g["W3"] = dH3.T @ H2
    g["b3"] = dH3.sum(0)
    dH2 = r((dH3 @ P["W3"]) * (H2 > 0))
    g["W2"] = dH2.T @ H1
    g["b2"] = dH2.sum(0)
    dH1 = r((dH2 @ P["W2"]) * (H1 > 0))
    g["W1"] = dH1.T @ X
    g["b1"] = dH1.sum(0)
    dX = dH1 @ P["W1"]
    genc = np.zeros_like(P["enc"])
    for l, (idx, wt) in enumerate(cs):
        for q in range(8):
            np.add.at(genc, idx[:, q], wt[:, q:q + 1] * dX[:, l * FEAT:(l + 1) * FEAT])
    g["enc"] = genc
    flat = np.zeros(L["total"])
    for n in ("enc", "W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"):
        o, sz = L[n]
        flat[o:o + sz] = g[n].reshape(-1)
    return loss, flat, L

"""CPU reference of the learned preconditioner (test oracle): the same
message-passing network, readout and losses (Hutchinson and the FSAI /
Kaporin objective) as the GPU kernels,
written with torch autograd in FP64.  The inputs of the layers' matrix
products are rounded to bfloat16 as the tensor-core kernels do; everything
else is FP64, so forward values and gradients agree with the GPU to the
FP32-accumulation level (forward) and to the BF16 rounding of the backward
operands (gradients)."""
import numpy as np
import torch

HID, FIN = 32, 16
KC0, KC = 2 * FIN, 2 * HID
OFF = {}
_o = 0
for name, size in (("W0", KC0 * HID), ("b0", HID), ("W1", KC * HID), ("b1", HID), ("W2", KC * HID), ("b2", HID),
                   ("rd", HID), ("ro", HID), ("ro2", HID)):
    OFF[name] = (_o, size)
    _o += size
NPARAM = _o


def bf16(t):
    return t.to(torch.bfloat16).to(torch.float64)


def unpack(p):
    out = {}
    for name, (o, s) in OFF.items():
        v = p[o:o + s]
        if name.startswith("W"):
            v = v.reshape(-1, HID)
        out[name] = v
    return out


def hop2(rowptr, col, what):
    """The two-hop pattern (j at distance exactly two, both triangles) in the
    GPU's enumeration order, with path weights pw_ij = sum_k what_ik what_kj
    (FP32 products, FP32 fused accumulation) and transposed positions."""
    n = len(rowptr) - 1
    rows, cols, pws = [], [], []
    rp = [0]
    for i in range(n):
        a, b = rowptr[i], rowptr[i + 1]
        nb1 = set(int(c) for c in col[a:b])
        qj, qw = [], []
        for k1 in range(a, b):
            k = int(col[k1])
            for k2 in range(rowptr[k], rowptr[k + 1]):
                j = int(col[k2])
                if j == i or j in nb1:
                    continue
                prod = np.float64(what[k1]) * np.float64(what[k2])
                if j in qj:
                    s_ = qj.index(j)
                    qw[s_] = np.float32(prod + np.float64(qw[s_]))
                else:
                    qj.append(j)
                    qw.append(np.float32(prod))
        rows += [i] * len(qj)
        cols += qj
        pws += qw
        rp.append(len(cols))
    rp = np.array(rp, np.int64)
    cols = np.array(cols, np.int64)
    pos = {(int(r), int(c)): e for e, (r, c) in enumerate(zip(rows, cols))}
    rev = np.array([pos.get((int(c), int(r)), -1) for r, c in zip(rows, cols)], np.int64)
    return rp, np.array(rows, np.int64), cols, np.array(pws, np.float32), rev


def prepare(rowptr, col, w, diag, adiag, hops=1):
    """what, dh, features as the GPU computes them (FP32), as float64 tensors."""
    n = len(diag)
    ri = np.repeat(np.arange(n), np.diff(rowptr))
    dh = (1.0 / np.sqrt(adiag)).astype(np.float32)
    what = (w.astype(np.float32) * dh[ri]) * dh[col]
    X = np.zeros((n, FIN), np.float32)
    X[:, 0] = 1.0
    X[:, 1] = (diag / adiag).astype(np.float32)
    s = np.zeros(n, np.float32)
    m = np.zeros(n, np.float32)
    sl = np.zeros(n, np.float32)
    ml = np.zeros(n, np.float32)
    nl = np.zeros(n, np.float32)
    for i in range(n):
        a, b = rowptr[i], rowptr[i + 1]
        s[i] = np.float32(0)
        for k in range(a, b):
            s[i] = np.float32(s[i] + what[k])
            if col[k] < i:
                sl[i] = np.float32(sl[i] + what[k])
                ml[i] = max(ml[i], what[k])
                nl[i] += 1
        m[i] = what[a:b].max() if b > a else 0.0
    X[:, 2] = s
    X[:, 3] = m
    X[:, 4] = (np.diff(rowptr).astype(np.float32)) * np.float32(0.125)
    X[:, 5] = sl
    X[:, 6] = nl * np.float32(0.125)
    X[:, 7] = ml
    T = lambda a: torch.from_numpy(np.asarray(a, np.float64))
    nnz = len(col)
    if hops == 2:
        rp2, ri2, col2, pw, rev2 = hop2(rowptr, col, what)
    else:
        rp2, ri2, col2, pw, rev2 = (np.zeros(n + 1, np.int64), np.zeros(0, np.int64), np.zeros(0, np.int64),
                                    np.zeros(0, np.float32), np.zeros(0, np.int64))
    # triples (entry of m, weight, entry of j) of tr(Gt What Gt^T) = sum_i sum_{m,j in S_i} Gt_im what_mj Gt_ij,
    # entries indexed into cat([gd, gl, gl2]) (gd: 0..n-1, gl: n + CSR position, gl2: n + nnz + two-hop position)
    tm, tw, tj = [], [], []
    pos = {}
    for i in range(n):
        for k in range(rowptr[i], rowptr[i + 1]):
            pos[(i, int(col[k]))] = k
    for i in range(n):
        mem = [(i, i)] + [(int(col[k]), n + k) for k in range(rowptr[i], rowptr[i + 1]) if col[k] < i]
        mem += [(int(col2[e]), n + nnz + e) for e in range(rp2[i], rp2[i + 1]) if col2[e] < i]
        for (m_, em) in mem:
            for (j_, ej) in mem:
                if m_ != j_ and (m_, j_) in pos:
                    tm.append(em)
                    tw.append(what[pos[(m_, j_)]])
                    tj.append(ej)
    return dict(n=n, ri=torch.from_numpy(ri), col=torch.from_numpy(col.astype(np.int64)), what=T(what), dh=T(dh),
                X=T(X), tm=torch.tensor(tm, dtype=torch.int64), tw=T(np.asarray(tw, np.float32)),
                tj=torch.tensor(tj, dtype=torch.int64), hops=hops, rp2=rp2, ri2=torch.from_numpy(ri2),
                col2=torch.from_numpy(col2), pw=T(pw))


def agg(G, H):
    out = torch.zeros_like(H)
    return out.index_add(0, G["ri"], G["what"][:, None] * H[G["col"]])


def layer(G, H, W, b, res):
    Xcat = torch.cat([H, agg(G, H)], dim=1)
    Z = bf16(Xcat) @ bf16(W) + b
    return (H if res else 0.0) + torch.relu(Z)


def factor(G, params, store_bf16=False):
    """store_bf16: the hidden features rounded to bfloat16 after each layer,
    as the per-step factor (inference) stores them."""
    P = unpack(params)
    keep = bf16 if store_bf16 else (lambda t: t)
    H1 = keep(layer(G, G["X"], P["W0"], P["b0"], False))
    H2 = keep(layer(G, H1, P["W1"], P["b1"], True))
    H3 = keep(layer(G, H2, P["W2"], P["b2"], True))
    gd = 1.0 + H3 @ P["rd"]
    lower = G["col"] < G["ri"]
    gl = G["what"] * ((H3[G["ri"]] * H3[G["col"]]) @ P["ro"])
    gl = torch.where(lower, gl, torch.zeros_like(gl))
    if G["hops"] == 2:
        lower2 = G["col2"] < G["ri2"]
        gl2 = G["pw"] * ((H3[G["ri2"]] * H3[G["col2"]]) @ P["ro2"])
        G["gl2"] = torch.where(lower2, gl2, torch.zeros_like(gl2))
    else:
        G["gl2"] = torch.zeros(0, dtype=torch.float64)
    return gd, gl


def apply_G(G, gd, gl, v):
    lower = G["col"] < G["ri"]
    out = gd * v
    return out.index_add(0, G["ri"][lower], gl[lower] * v[G["col"][lower]])


def apply_GT(G, gd, gl, v):
    lower = G["col"] < G["ri"]
    out = gd * v
    return out.index_add(0, G["col"][lower], gl[lower] * v[G["ri"][lower]])


def apply_At(G, v):
    out = v.clone()
    return out.index_add(0, G["ri"], -G["what"] * v[G["col"]])


def loss(G, params, probes):
    gd, gl = factor(G, params)
    tot = 0.0
    for z in probes:
        r = apply_G(G, gd, gl, apply_At(G, apply_GT(G, gd, gl, z))) - z
        tot = tot + (r * r).sum()
    return tot / (len(probes) * G["n"])


def loss_kaporin(G, params):
    """(1/n) [tr(Gt At Gt^T) - 2 sum log Gt_ii], At = I - What."""
    gd, gl = factor(G, params)
    e = torch.cat([gd, gl, G["gl2"]])
    tr = (e * e).sum() - (e[G["tm"]] * G["tw"] * e[G["tj"]]).sum()
    return (tr - 2.0 * torch.log(gd).sum()) / G["n"]


def loss_and_grad(rowptr, col, w, diag, adiag, params, probes, hops=1):
    """probes None: the Kaporin objective; else the Hutchinson loss."""
    G = prepare(rowptr, col, w, diag, adiag, hops)
    p = torch.tensor(np.asarray(params, np.float64), requires_grad=True)
    if probes is None:
        L = loss_kaporin(G, p)
        L.backward()
        return float(L.detach()), p.grad.numpy().copy()
    z = [torch.from_numpy(np.asarray(q, np.float64)) for q in probes]
    L = loss(G, p, z)
    L.backward()
    return float(L.detach()), p.grad.numpy().copy()


def forward_values(rowptr, col, w, diag, adiag, params, hops=1, store_bf16=True):
    """The factor as lv_learn_factor computes it (the per-step inference,
    hidden features stored in bfloat16)."""
    G = prepare(rowptr, col, w, diag, adiag, hops)
    with torch.no_grad():
        gd, gl = factor(G, torch.tensor(np.asarray(params, np.float64)), store_bf16)
    if hops == 2:
        return gd.numpy(), gl.numpy(), G["X"].numpy(), (G["rp2"], G["col2"].numpy(), G["gl2"].numpy())
    return gd.numpy(), gl.numpy(), G["X"].numpy()

"""CPU oracle of the learned preconditioner (TEST INFRASTRUCTURE ONLY).

Only the tests (and nothing on the product path) use this module.  It is a
float64 numpy restatement of the network, the preconditioner application and
the training loss of neopz_gb300/csrc/gpz_learned.cu, with an analytic
backward pass.  The GPU forward / backward kernels are checked against it,
and it is itself checked against central finite differences
(tests/test_oracle_golden.py).  The learned preconditioner has no counterpart
in the reference; the matrix and load vectors it is trained on come from the
oracle's restatement of the reference's assembly.

Network (H = 32): h0 = tanh(W0 x + b0), x = log(coefficient); for l = 1, 2:
n_c = mean of h over the elements at connect c, nb_e = mean of n over the
element's connects, h += tanh(W_l [h; nb] + b_l); F_e = Wo h2 + bo, reshaped
NS x R.  M r = S (alpha u + m * sum_e Q_e^T F_e F_e^T Q_e (m * u)), u = S r,
S = diag(A)^-1/2, m = 0 on penalty-Dirichlet equations, alpha = exp(a).
Loss = mean_j (M r_j - e_j)^T A (M r_j - e_j) / e_j^T A e_j on masked vectors.
"""
import numpy as np

H = 32


def layout(NS, R):
    NR = NS * R
    o, off = 0, {}
    for name, size in (("W0", H), ("b0", H), ("W1", H * 2 * H), ("b1", H), ("W2", H * 2 * H), ("b2", H),
                       ("Wo", NR * H), ("bo", NR), ("a", 1)):
        off[name] = (o, size)
        o += size
    return off, o


def unpack(p, NS, R):
    off, _ = layout(NS, R)
    g = {k: np.asarray(p[a:a + n], np.float64) for k, (a, n) in off.items()}
    g["W1"] = g["W1"].reshape(H, 2 * H)
    g["W2"] = g["W2"].reshape(H, 2 * H)
    g["Wo"] = g["Wo"].reshape(NS * R, H)
    return g


def pack(g, NS, R):
    off, n = layout(NS, R)
    p = np.zeros(n)
    for k, (a, m) in off.items():
        p[a:a + m] = np.asarray(g[k]).reshape(-1)
    return p


class Mesh:
    """Incidence of the volume elements: ec[E][nsides] connects, dest[E][NS] equations."""

    def __init__(self, ec, dest, nconn, mask, diag, feat):
        self.ec = np.asarray(ec, np.int64)
        self.dest = np.asarray(dest, np.int64)
        self.E, self.nsides = self.ec.shape
        self.NS = self.dest.shape[1]
        self.nconn = nconn
        self.mask = np.asarray(mask, np.float64)
        self.dsq = 1.0 / np.sqrt(np.asarray(diag, np.float64))
        self.feat = np.asarray(feat, np.float64)
        self.cnt = np.bincount(self.ec.reshape(-1), minlength=nconn).astype(np.float64)

    def node_mean(self, h):
        s = np.zeros((self.nconn, h.shape[1]))
        np.add.at(s, self.ec.reshape(-1), np.repeat(h, self.nsides, axis=0))
        return np.where(self.cnt[:, None] > 0, s / np.maximum(self.cnt, 1)[:, None], 0.0)

    def elem_mean(self, nm):
        return nm[self.ec].mean(axis=1)


def forward(mesh, p, R):
    g = unpack(p, mesh.NS, R)
    act = {}
    h0 = np.tanh(np.outer(mesh.feat, g["W0"]) + g["b0"])
    act["h0"] = h0
    h = h0
    for l in (1, 2):
        nb = mesh.elem_mean(mesh.node_mean(h))
        y = np.tanh(np.concatenate([h, nb], 1) @ g[f"W{l}"].T + g[f"b{l}"])
        act[f"in{l}"] = np.concatenate([h, nb], 1)
        act[f"y{l}"] = y
        h = h + y
        act[f"h{l}"] = h
    F = (h @ g["Wo"].T + g["bo"]).reshape(mesh.E, mesh.NS, R)
    return F, act


def apply_M(mesh, F, r, alpha=1.0):
    u = mesh.dsq * r
    um = mesh.mask * u
    ue = um[mesh.dest]                          # E x NS
    t = np.einsum("eir,ei->er", F, ue)
    ce = np.einsum("eir,er->ei", F, t)
    c = np.zeros_like(r)
    np.add.at(c, mesh.dest.reshape(-1), ce.reshape(-1))
    return mesh.dsq * (alpha * u + mesh.mask * c)


def loss_and_grad(mesh, A, p, R, Rs, Es):
    """A: scipy sparse matrix; Rs, Es: [P][n] residuals and errors."""
    F, act = forward(mesh, p, R)
    g = unpack(p, mesh.NS, R)
    alpha = float(np.exp(g["a"][0]))
    P = len(Rs)
    loss = 0.0
    da = 0.0
    dF = np.zeros_like(F)
    for r, e in zip(Rs, Es):
        em = mesh.mask * e
        eAe = em @ (A @ em)
        z = apply_M(mesh, F, r, alpha)
        w = mesh.mask * (z - e)
        aw = A @ w
        loss += (w @ aw) / eAe / P
        gz = 2.0 / (P * eAe) * mesh.mask * aw
        da += alpha * (gz @ (mesh.dsq ** 2 * r))
        ue = (mesh.mask * mesh.dsq * r)[mesh.dest]
        ge = (mesh.mask * mesh.dsq * gz)[mesh.dest]
        t = np.einsum("eir,ei->er", F, ue)
        s = np.einsum("eir,ei->er", F, ge)
        dF += ge[:, :, None] * t[:, None, :] + ue[:, :, None] * s[:, None, :]
    dFf = dF.reshape(mesh.E, -1)
    grad = {}
    grad["Wo"] = dFf.T @ act["h2"]
    grad["bo"] = dFf.sum(0)
    dh = dFf @ g["Wo"]
    for l in (2, 1):
        y = act[f"y{l}"]
        dpre = dh * (1 - y * y)
        grad[f"W{l}"] = dpre.T @ act[f"in{l}"]
        grad[f"b{l}"] = dpre.sum(0)
        gin = dpre @ g[f"W{l}"]
        dh = dh + gin[:, :H]
        dnb = gin[:, H:]
        # transpose of nb = elem_mean(node_mean(h))
        dnm = np.zeros((mesh.nconn, H))
        np.add.at(dnm, mesh.ec.reshape(-1), np.repeat(dnb / mesh.nsides, mesh.nsides, axis=0))
        dh = dh + (dnm / np.maximum(mesh.cnt, 1)[:, None])[mesh.ec].sum(axis=1)
    h0 = act["h0"]
    dpre0 = dh * (1 - h0 * h0)
    grad["W0"] = dpre0.T @ mesh.feat
    grad["b0"] = dpre0.sum(0)
    grad["a"] = np.array([da])
    return loss, pack(grad, mesh.NS, R)


def loss_only(mesh, A, p, R, Rs, Es):
    F, _ = forward(mesh, p, R)
    alpha = float(np.exp(unpack(p, mesh.NS, R)["a"][0]))
    P = len(Rs)
    loss = 0.0
    for r, e in zip(Rs, Es):
        em = mesh.mask * e
        z = apply_M(mesh, F, r, alpha)
        w = mesh.mask * (z - e)
        loss += (w @ (A @ w)) / (em @ (A @ em)) / P
    return loss


def mesh_from_oracle(om, A, coef):
    """Incidence of an oracle mesh (volume elements in element order; Dirichlet equations masked)."""
    ec, dest = [], []
    mask = np.ones(om.neq)
    for e in range(om.ncel):
        c = om.cel(e)
        if c["is_bc"]:
            mask[c["dest"]] = 0.0
            continue
        ec.append(c["conn"])
        dest.append(c["dest"])
    return Mesh(np.array(ec), np.array(dest), om.nconnects, mask, A.diagonal(), np.log(coef))

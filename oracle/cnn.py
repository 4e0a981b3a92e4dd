"""CPU oracle of the gauge-covariant preconditioner network (test infrastructure only).

numpy, complex128, canonical site order.  Semantics (the same as chroma_gb300/csrc/cnn.cu):

    out(x)[o][a] = sum_{d=0..8} sum_i W_d[o][i] (T_d h)(x)[i][a]
    T_0 h(x) = h(x),  T_{1+2mu} h(x) = U_mu(x) h(x+mu),  T_{2+2mu} h(x) = U_mu(x-mu)^dag h(x-mu)

The input is an odd-site spinor used as 4 channels (spins) with the even sites zeroed, the
output the last layer's odd sites.  Loss: sum_b |K(r_b) - e_b|^2 / |e_b|^2 over odd sites.
Gradients are dL/dRe W + i dL/dIm W, computed by the analytic backward pass and checked
against finite differences in tests/test_cnn_oracle.py.  No reference counterpart: parity
of the learned preconditioner is pinned only by these identities.
"""
import numpy as np


def _coords(dims):
    V = int(np.prod(dims))
    s = np.arange(V)
    x = s % dims[0]
    y = (s // dims[0]) % dims[1]
    z = (s // (dims[0] * dims[1])) % dims[2]
    t = s // (dims[0] * dims[1] * dims[2])
    return np.stack([x, y, z, t], axis=1)


class CnnOracle:
    def __init__(self, dims, links):
        self.dims = tuple(dims)
        self.V = int(np.prod(dims))
        self.u = np.asarray(links, dtype=np.complex128).reshape(self.V, 4, 3, 3)
        X = _coords(dims)
        self.odd = (X.sum(axis=1) % 2) == 1
        self.fwd, self.bwd = [], []
        for mu in range(4):
            for sgn, lst in ((1, self.fwd), (-1, self.bwd)):
                Y = X.copy()
                Y[:, mu] = (Y[:, mu] + sgn) % dims[mu]
                lst.append(Y[:, 0] + dims[0] * (Y[:, 1] + dims[1] * (Y[:, 2] + dims[2] * Y[:, 3])))

    def T(self, h, d):
        if d == 0:
            return h
        mu, back = (d - 1) // 2, (d - 1) % 2 == 1
        if not back:
            return np.einsum("xab,xib->xia", self.u[:, mu], h[self.fwd[mu]])
        n = self.bwd[mu]
        return np.einsum("xba,xib->xia", np.conj(self.u[n, mu]), h[n])

    def T_adj(self, q, d):
        if d == 0:
            return q
        mu, back = (d - 1) // 2, (d - 1) % 2 == 1
        if not back:  # (T_{+mu}^dag q)(y) = U_mu(y-mu)^dag q(y-mu)
            n = self.bwd[mu]
            return np.einsum("xba,xib->xia", np.conj(self.u[n, mu]), q[n])
        # (T_{-mu}^dag q)(y) = U_mu(y) q(y+mu)
        return np.einsum("xab,xib->xia", self.u[:, mu], q[self.fwd[mu]])

    def layer(self, h, W):
        return sum(np.einsum("oi,xia->xoa", W[d], self.T(h, d)) for d in range(9))

    def embed(self, v):
        h = np.asarray(v, dtype=np.complex128).reshape(self.V, 4, 3).copy()
        h[~self.odd] = 0
        return h

    def forward(self, v, Ws):
        acts = [self.embed(v)]
        for W in Ws:
            acts.append(self.layer(acts[-1], W))
        return acts

    def apply(self, v, Ws):
        y = self.forward(v, Ws)[-1].copy()
        y[~self.odd] = 0
        return y

    def loss_grad(self, vs, es, Ws):
        loss = 0.0
        grads = [np.zeros_like(W) for W in Ws]
        for v, e in zip(vs, es):
            e = np.asarray(e, dtype=np.complex128).reshape(self.V, 4, 3)
            acts = self.forward(v, Ws)
            en = np.sum(np.abs(e[self.odd]) ** 2)
            r = acts[-1] - e
            r[~self.odd] = 0
            loss += np.sum(np.abs(r) ** 2) / en
            delta = 2.0 * r / en
            for li in range(len(Ws) - 1, -1, -1):
                W = Ws[li]
                for d in range(9):
                    grads[li][d] += np.einsum("xoa,xia->oi", delta, np.conj(self.T(acts[li], d)))
                if li > 0:
                    delta = sum(self.T_adj(np.einsum("oi,xoa->xia", np.conj(W[d]), delta), d) for d in range(9))
        return loss, grads


def unpack_weights(flat, hidden=12, layers=4):
    """Interleaved (re, im) floats of gbc_precond_weights -> list of (9, cout, cin) complex arrays."""
    flat = np.asarray(flat, dtype=np.float64)
    z = flat[0::2] + 1j * flat[1::2]
    Ws, k = [], 0
    for l in range(layers):
        ci = 4 if l == 0 else hidden
        co = 4 if l == layers - 1 else hidden
        n = 9 * co * ci
        Ws.append(z[k:k + n].reshape(9, co, ci))
        k += n
    return Ws


def pack_weights(Ws):
    z = np.concatenate([W.reshape(-1) for W in Ws])
    out = np.empty(2 * z.size, dtype=np.float32)
    out[0::2] = z.real
    out[1::2] = z.imag
    return out

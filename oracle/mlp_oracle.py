"""numpy FP64 restatement of the learned SGS closure (no reference counterpart).

TEST INFRASTRUCTURE ONLY: the tests use it to check the library's MLP kernels (forward,
backward, AdamW, features, BF16 inference); the library never calls it.

Model: x (10 features) -> h1 = gelu(W1 x + b1) (64) -> h2 = gelu(W2 h1 + b2) (64)
-> z = w3 . h2 + b3 -> Cs2 = softplus(z).  gelu is the tanh form
0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))).  Loss = mean((Cs2 - y)^2).
Features at a point (from the 9 velocity gradients duidxj, igrid order): the gradients
divided by |S| = sqrt(2 Sij Sij) (0 where |S| = 0), and ln(1 + Delta/eta) with the local
Kolmogorov estimate eta = (nu^3 / (nu |S|^2))^(1/4), i.e. Delta/eta = Delta sqrt(|S|/nu).
The eddy viscosity is nu_sgs = Cs2 Delta^2 |S|.
Parameters are one flat float array: W1 (64x10, row-major), b1 (64), W2 (64x64), b2 (64),
w3 (64), b3 (1) -- 4929 values.
"""
import numpy as np

NIN, NH = 10, 64
SIZES = [("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("w3", (NH,)), ("b3", (1,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)
C_GELU = np.sqrt(2.0 / np.pi)


def unpack(p):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SIZES])


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(C_GELU * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(C_GELU * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * C_GELU * (1.0 + 3 * 0.044715 * x * x)


def softplus(z):
    return np.logaddexp(0.0, z)


def sigmoid(z):
    return 0.5 * (1.0 + np.tanh(0.5 * z))


def forward(p, X):
    w = unpack(p)
    z1 = X @ w["W1"].T + w["b1"]
    h1 = gelu(z1)
    z2 = h1 @ w["W2"].T + w["b2"]
    h2 = gelu(z2)
    z3 = h2 @ w["w3"] + w["b3"][0]
    return softplus(z3), (z1, h1, z2, h2, z3)


def loss_and_grad(p, X, y):
    """Mean squared error of Cs2 against y and its gradient with respect to p."""
    w = unpack(p)
    cs2, (z1, h1, z2, h2, z3) = forward(p, X)
    B = X.shape[0]
    r = cs2 - y
    loss = np.mean(r * r)
    dz3 = (2.0 / B) * r * sigmoid(z3)
    g = {"b3": np.array([dz3.sum()]), "w3": h2.T @ dz3}
    dz2 = np.outer(dz3, w["w3"]) * gelu_grad(z2)
    g["W2"] = dz2.T @ h1
    g["b2"] = dz2.sum(axis=0)
    dz1 = (dz2 @ w["W2"]) * gelu_grad(z1)
    g["W1"] = dz1.T @ X
    g["b1"] = dz1.sum(axis=0)
    return loss, pack(g)


def adamw(p, g, m, v, t, lr, wd, b1=0.9, b2=0.999, eps=1e-8):
    """One AdamW update (decoupled weight decay); returns new (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    p = p - lr * (mh / (np.sqrt(vh) + eps) + wd * p)
    return p, m, v


def features(d, delta, nu):
    """Features of every point from the 9 gradient arrays (any common shape) -> (n, 10)."""
    S = [d[0], 0.5 * (d[1] + d[3]), 0.5 * (d[2] + d[6]), d[4], 0.5 * (d[5] + d[7]), d[8]]
    s = S[0] * S[0] + 2 * S[1] * S[1] + 2 * S[2] * S[2] + S[3] * S[3] + 2 * S[4] * S[4] + S[5] * S[5]
    mag = np.sqrt(2.0 * s).ravel(order="F")
    X = np.zeros((mag.size, NIN))
    inv = np.where(mag > 0, 1.0 / np.where(mag > 0, mag, 1.0), 0.0)
    for i in range(9):
        X[:, i] = np.asarray(d[i]).ravel(order="F") * inv
    X[:, 9] = np.log1p(delta * np.sqrt(mag / nu))
    return X, mag


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(x, dtype=np.float32).copy()
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def infer_bf16(p, X):
    """The inference kernel's arithmetic: BF16 inputs, weights and activations (both hidden
    layers and w3), FP32-exact products, FP64 sums standing in for FP32 accumulation.  The
    kernel evaluates GELU in BF16 arithmetic with an approximate tanh; here GELU is exact and
    rounded once, so the two differ by a few BF16 ulps per activation."""
    w = unpack(p)
    xb = bf16(X)
    z1 = xb @ bf16(w["W1"]).T + np.asarray(w["b1"], dtype=np.float32)
    h1 = bf16(gelu(z1))
    z2 = h1 @ bf16(w["W2"]).T + np.asarray(w["b2"], dtype=np.float32)
    h2 = bf16(gelu(z2))
    z3 = h2 @ bf16(np.asarray(w["w3"], dtype=np.float32)) + np.float32(w["b3"][0])
    return softplus(z3)

"""CPU reference of the selector network (test infrastructure only).

Same parameter layout and maths as fmm_gb300/csrc/mlp.cuh: normalised inputs,
three ReLU layers, linear output; loss = mean squared error over samples and
outputs.  Used to check the GPU forward pass and gradients.
"""
import numpy as np

IN, H, OUT = 17, 64, 11


def offsets():
    o = {}
    k = 0
    for name, size in (("mean", IN), ("istd", IN), ("W1", H * IN), ("b1", H), ("W2", H * H), ("b2", H),
                       ("W3", H * H), ("b3", H), ("W4", OUT * H), ("b4", OUT)):
        o[name] = (k, size)
        k += size
    o["total"] = k
    return o


def unpack(p):
    o = offsets()
    g = lambda n: np.asarray(p[o[n][0]:o[n][0] + o[n][1]], dtype=np.float64)
    return dict(mean=g("mean"), istd=g("istd"), W1=g("W1").reshape(H, IN), b1=g("b1"),
                W2=g("W2").reshape(H, H), b2=g("b2"), W3=g("W3").reshape(H, H), b3=g("b3"),
                W4=g("W4").reshape(OUT, H), b4=g("b4"))


def forward(p, X):
    q = unpack(p)
    a0 = (X - q["mean"]) * q["istd"]
    z1 = a0 @ q["W1"].T + q["b1"]
    a1 = np.maximum(z1, 0)
    z2 = a1 @ q["W2"].T + q["b2"]
    a2 = np.maximum(z2, 0)
    z3 = a2 @ q["W3"].T + q["b3"]
    a3 = np.maximum(z3, 0)
    y = a3 @ q["W4"].T + q["b4"]
    return y, (a0, a1, a2, a3)


def loss_and_grad(p, X, Y):
    """Mean squared error and its gradient (flat, same layout as p)."""
    q = unpack(p)
    y, (a0, a1, a2, a3) = forward(p, X)
    n = X.shape[0]
    r = y - Y
    loss = float(np.mean(r ** 2))
    d4 = 2 * r / (n * OUT)
    d3 = (d4 @ q["W4"]) * (a3 > 0)
    d2 = (d3 @ q["W3"]) * (a2 > 0)
    d1 = (d2 @ q["W2"]) * (a1 > 0)
    g = np.zeros(offsets()["total"])
    o = offsets()

    def put(name, val):
        g[o[name][0]:o[name][0] + o[name][1]] = val.reshape(-1)

    put("W4", d4.T @ a3)
    put("b4", d4.sum(0))
    put("W3", d3.T @ a2)
    put("b3", d3.sum(0))
    put("W2", d2.T @ a1)
    put("b2", d2.sum(0))
    put("W1", d1.T @ a0)
    put("b1", d1.sum(0))
    return loss, g


def init_params(X, seed=0):
    """He-initialised weights, zero biases, normalisation from X."""
    rng = np.random.default_rng(seed)
    o = offsets()
    p = np.zeros(o["total"], dtype=np.float32)
    mean = X.mean(0)
    std = X.std(0)
    std[std < 1e-6] = 1.0
    p[o["mean"][0]:o["mean"][0] + IN] = mean
    p[o["istd"][0]:o["istd"][0] + IN] = 1.0 / std
    for name, fan_in in (("W1", IN), ("W2", H), ("W3", H), ("W4", H)):
        a, n = o[name]
        p[a:a + n] = rng.normal(0.0, np.sqrt(2.0 / fan_in), n)
    return p

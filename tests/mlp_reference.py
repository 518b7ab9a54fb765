"""float64 numpy reference of the surrogate MLP (test infrastructure): the
same network as sfsim_gb300's kernels, with BF16 rounding applied at the
same points (features, hidden activations and their gradients, the BF16
weight copies), so that its gradients check the GPU's forward and backward
GEMMs."""
import numpy as np

N_SMOOTH, N_PHASES = 6, 4
N_COORDS = N_SMOOTH + N_PHASES
N_IN, N_HID = 32 * N_SMOOTH + 16 * N_PHASES, 256
N_OUT = 4  # three log-space corrections to the table lookup and a log variance
SHAPES = [(N_HID, N_IN), (N_HID, N_HID), (N_HID, N_HID), (N_HID, N_HID), (N_OUT, N_HID)]
VAR_WEIGHT = 0.01


def bf16(x):
    """Round to bfloat16 (nearest even) and return as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    out, o = [], 0
    for (r, c) in SHAPES:
        W = params[o:o + r * c].reshape(r, c).astype(np.float64)
        o += r * c
        b = params[o:o + r].astype(np.float64)
        o += r
        out.append((W, b))
    return out


def features(coords):
    """Smooth coordinates: 16 frequencies 2^(k/2); cell phases: 8 harmonics 2 (k + 1);
    sin and cos of pi f u, in coordinate order."""
    n = coords.shape[0]
    k = np.arange(16)
    f = np.where(k % 2 == 1, np.float32(np.sqrt(2.0)), 1.0) * 2.0 ** (k // 2)
    ang = np.pi * coords[:, :N_SMOOTH, None].astype(np.float64) * f[None, None, :]
    smooth = np.stack([np.sin(ang), np.cos(ang)], axis=-1).reshape(n, 32 * N_SMOOTH)
    h = 2.0 * (np.arange(8) + 1)
    angp = np.pi * coords[:, N_SMOOTH:, None].astype(np.float64) * h[None, None, :]
    phase = np.stack([np.sin(angp), np.cos(angp)], axis=-1).reshape(n, 16 * N_PHASES)
    return np.concatenate([smooth, phase], axis=1)


def silu(z):
    return z / (1 + np.exp(-z))


def dsilu(z):
    s = 1 / (1 + np.exp(-z))
    return s * (1 + z * (1 - s))


N_COND = 8  # atmosphere inputs of the conditioned network


def cond_term(params, groups, inputs):
    """First-layer term U g of each row of a conditioned network (U [256][8]
    after the plain parameters), or 0 for a plain parameter vector."""
    n_plain = sum(r * c + r for (r, c) in SHAPES)
    if params.size == n_plain:
        return 0.0
    U = params[n_plain:].reshape(N_HID, N_COND).astype(np.float64)
    return inputs.astype(np.float64)[groups] @ U.T


def loss_and_grads(params, coords, targets, var_weight=VAR_WEIGHT, groups=None, inputs=None):
    """Mean squared error of the corrections (the reported loss) with the
    Gaussian negative log-likelihood of the squared error under the predicted
    variance exp(s) added to the gradients, weighted by var_weight.  With
    `groups` and `inputs` the network is the conditioned one: row i adds
    U inputs[groups[i]] to the first layer."""
    layers = unpack(params)
    n = coords.shape[0]
    H = [bf16(features(coords))]
    Z = []
    for l in range(4):
        W, b = layers[l]
        z = H[-1] @ bf16(W).T + b
        if l == 0 and groups is not None:
            z = z + cond_term(params, groups, inputs)
        Z.append(z)
        H.append(bf16(silu(z)))
    W5, b5 = layers[4]
    out = H[4] @ W5.T + b5
    e = out[:, :3] - targets
    m = np.mean(e * e, axis=1)
    loss = np.mean(m)
    s = np.clip(out[:, 3], -40, 20)
    dout = np.concatenate([2 * e / (3 * n), (var_weight * 0.5 * (1 - m * np.exp(-s)) / n)[:, None]], axis=1)
    grads = []
    dW5 = dout.T @ H[4]
    db5 = dout.sum(axis=0)
    dZ = bf16((dout @ W5) * dsilu(Z[3]))
    g = [None] * 5
    g[4] = (dW5, db5)
    dU = None
    for l in range(3, -1, -1):
        W, b = layers[l]
        dW = dZ.T @ H[l]
        db = dZ.sum(axis=0)
        g[l] = (dW, db)
        if l == 0 and groups is not None:
            dU = dZ.T @ inputs.astype(np.float64)[groups]
        if l > 0:
            dZ = bf16((dZ @ bf16(W)) * dsilu(Z[l - 1]))
    for (dW, db) in g:
        grads.append(dW.ravel())
        grads.append(db.ravel())
    if dU is not None:
        grads.append(dU.ravel())
    return loss, np.concatenate(grads)


def forward(params, coords, inputs=None):
    """Network outputs [n][4] (three corrections, log variance) for coords
    [n][4], with the GPU's BF16 roundings; `inputs` [8] are the atmosphere
    inputs of a conditioned network."""
    layers = unpack(params)
    H = bf16(features(coords))
    for l in range(4):
        W, b = layers[l]
        if l == 0 and inputs is not None:
            b = b + cond_term(params, np.zeros(1, np.int64), np.asarray(inputs)[None, :])[0]
        H = bf16(silu(H @ bf16(W).T + b))
    W5, b5 = layers[4]
    return H @ W5.T + b5

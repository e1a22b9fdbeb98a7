"""TEST INFRASTRUCTURE -- CPU restatement of the learned surrogate (numpy, FP64).

Checks the GPU training kernels (forward, backward, loss) and the tensor-core inference of
libsps_gb300.so, and the tuples the GPU captures from the Drucker-Prager flow rule.  Only
tests/ and the benchmark's checks import it.

  forward / loss_grad   the 14-128-128-128-4 SiLU network of include/sps_surrogate.h with
                        the same parameter layout; with quantize=True weights, inputs and
                        hidden activations are rounded to BF16 (round to nearest even) as
                        the GPU forward does, and gradients pass the rounding straight
                        through
  dp_target             the plastic source of drucker_prager
                        (code/3_SPH_material_2018.f90:2027-2039 of the Drucker-Prager
                        example) expressed in the scale-free tuple variables
  features              the tuple inputs from a stress, grad_u and the material
"""
import numpy as np

NIN, NOUT, H = 14, 4, 128
W1, B1 = 0, 16 * H
W2, B2 = B1 + H, B1 + H + H * H
W3, B3 = B2 + H, B2 + H + H * H
W4, B4 = B3 + H, B3 + H + H * 8
NPARAM = B4 + 8
LAYERS = [(W1, 16, H), (W2, H, H), (W3, H, H), (W4, H, 8)]


def bf16(a):
    """Round to BF16 (nearest even) through FP32, returned as float64."""
    f = np.asarray(a, np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, np.float64)
    out = []
    for off, k, n in LAYERS:
        out.append((p[off:off + k * n].reshape(k, n), p[off + k * n:off + k * n + n]))
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def forward(params, x, quantize=False):
    """Outputs (n x 4) and the cache of the pass."""
    q = bf16 if quantize else (lambda v: np.asarray(v, np.float64))
    n = len(x)
    a = np.zeros((n, 16))
    a[:, :NIN] = q(x)
    cache = [a]
    zs = []
    layers = unpack(params)
    for li, (W, b) in enumerate(layers):
        z = a @ q(W) + b
        if li < 3:
            zs.append(z)
            a = q(silu(z))
            cache.append(a)
        else:
            y = z
    return y[:, :NOUT], (cache, zs, layers)


def loss_grad(params, tuples, quantize=False):
    """Mean squared error over n rows x 4 outputs and its gradient (NPARAM)."""
    tuples = np.asarray(tuples, np.float64)
    x, t = tuples[:, :NIN], tuples[:, NIN:NIN + NOUT]
    y, (acts, zs, layers) = forward(params, x, quantize)
    n = len(x)
    d = y - t
    loss = float((d * d).sum() / (4.0 * n))
    dy = np.zeros((n, 8))
    dy[:, :NOUT] = 2.0 * d / (4.0 * n)
    q = bf16 if quantize else (lambda v: v)
    g = np.zeros(NPARAM)
    delta = dy
    for li in range(3, -1, -1):
        off, k, nn = LAYERS[li]
        W, _ = layers[li]
        a = acts[li]
        g[off:off + k * nn] = (a.T @ delta).ravel()
        g[off + k * nn:off + k * nn + nn] = delta.sum(axis=0)
        if li == 0:
            break
        dh = delta @ q(W).T
        z = zs[li - 1]
        s = 1.0 / (1.0 + np.exp(-z))
        delta = dh * (s * (1.0 + z * (1.0 - s)))
    return loss, g


def features(stress, grad_u, tanfi, coh, young, poiss, rho):
    """Tuple inputs (14) and the output scale G_mod |e| for one stress-point (FP64)."""
    s = np.asarray(stress, np.float64)
    gu = np.asarray(grad_u, np.float64)
    S = np.sqrt((s * s).sum())
    e11, e22 = gu[0], gu[3]
    e12 = 0.5 * (gu[2] + gu[1])
    w = 0.5 * (gu[2] - gu[1])
    en = np.sqrt(e11 * e11 + e22 * e22 + 2.0 * e12 * e12)
    x = np.array([*(s / S), e11 / en, e22 / en, e12 / en, 0.0, w / en, tanfi, coh / S, poiss,
                  np.log10(young) - 7.0, rho / 2000.0 - 1.0])
    return x, young / (2.0 * (1.0 + poiss)) * en


def dp_target(x):
    """Gs / (G_mod |e|) of the Drucker-Prager flow rule for tuple inputs x (n x 14)."""
    x = np.atleast_2d(np.asarray(x, np.float64))
    n = x[:, 0:4]
    sm = (n[:, 0] + n[:, 1] + n[:, 3]) / 3.0
    dn = np.stack([n[:, 0] - sm, n[:, 1] - sm, n[:, 2], n[:, 3] - sm], axis=1)
    sj = np.sqrt(dn[:, 2] ** 2 + 0.5 * (dn[:, 0] ** 2 + dn[:, 1] ** 2 + dn[:, 3] ** 2))
    e11, e22, e12 = x[:, 4], x[:, 5], x[:, 6]
    tanfi, nu = x[:, 9], x[:, 11]
    alpha = tanfi / np.sqrt(9.0 + 12.0 * tanfi * tanfi)
    k_over_g = 2.0 * (1.0 + nu) / (3.0 * (1.0 - 2.0 * nu))
    s_eps = dn[:, 0] * e11 + 2.0 * dn[:, 2] * e12 + dn[:, 1] * e22
    g2 = 3.0 * alpha * k_over_g * (e11 + e22) + s_eps / sj
    return -(dn / sj[:, None]) * g2[:, None]


def dp_source(stress, grad_u, tanfi, young, poiss):
    """Gs = -G of drucker_prager for a loading stress-point, in FP64 and physical units."""
    s = np.asarray(stress, np.float64)
    gu = np.asarray(grad_u, np.float64)
    sm = (s[0] + s[1] + s[3]) / 3.0
    dv = np.array([s[0] - sm, s[1] - sm, s[2], s[3] - sm])
    sj = np.sqrt(dv[2] ** 2 + 0.5 * (dv[0] ** 2 + dv[1] ** 2 + dv[3] ** 2))
    e11, e22, e12 = gu[0], gu[3], 0.5 * (gu[2] + gu[1])
    alpha = tanfi / np.sqrt(9.0 + 12.0 * tanfi * tanfi)
    gm = young / (2.0 * (1.0 + poiss))
    km = young / (3.0 * (1.0 - 2.0 * poiss))
    gs = gm / sj
    g2 = (3.0 * alpha * km * (e11 + e22) + gs * (dv[0] * e11 + 2.0 * dv[2] * e12 + dv[1] * e22)) / gm
    return -(gs * dv) * g2

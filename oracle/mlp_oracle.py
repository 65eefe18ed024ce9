"""ORACLE / TEST INFRASTRUCTURE ONLY: FP64 numpy statement of the learned surrogate.

The reference has no learned component; this module defines, in plain FP64 numpy, the
radial-descriptor MLP that the CUDA surrogate kernels implement; the tests compare the
kernels' forward pass, gradients and optimizer step with it:

  descriptor  G[i,k] = sum_{j != i} exp(-(r_ij - c_k)^2 / (2 w^2)),  32 centres c_k evenly
              spaced over [0.8, 3.0] sigma, width w = 0.1 sigma
  network     z1 = G W1 + b1, h1 = silu(z1)          (32 -> 64)
              z2 = h1 W2 + b2, h2 = silu(z2)         (64 -> 64)
              e  = h2 . w3 + b3                      (64 -> 1), per atom
  surrogate   E_s(config) = sum_i e_i
  loss        mean over configurations of (E_s - E_exact)^2
  update      Adam (Kingma & Ba 2015) with bias correction

`bf16` rounds to bfloat16 (round to nearest even) as the tensor-core forward pass sees
its operands (G, W1, h1, W2).
"""
import numpy as np

N_RBF, H1, H2 = 32, 64, 64
CENTRES = 0.8 + (3.0 - 0.8) * np.arange(N_RBF) / (N_RBF - 1)
WIDTH = 0.1


def bf16(x):
    """Round float values to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def descriptors(pos):
    """pos [N,3] -> G [N,32] in FP64."""
    d = pos[:, None, :] - pos[None, :, :]
    r = np.sqrt((d ** 2).sum(-1))
    np.fill_diagonal(r, np.inf)
    g = np.exp(-((r[:, :, None] - CENTRES[None, None, :]) ** 2) / (2 * WIDTH ** 2))
    return g.sum(axis=1)


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    return {
        "W1": rng.normal(0, 1 / np.sqrt(N_RBF), (N_RBF, H1)),
        "b1": np.zeros(H1),
        "W2": rng.normal(0, 1 / np.sqrt(H1), (H1, H2)),
        "b2": np.zeros(H2),
        "w3": rng.normal(0, 1 / np.sqrt(H2), H2),
        "b3": np.zeros(1),
    }


def forward(G, p, emulate_bf16=True):
    """G [rows,32] -> per-row energies and the intermediates."""
    q = (lambda x: bf16(x)) if emulate_bf16 else (lambda x: x)
    z1 = q(G) @ q(p["W1"]) + p["b1"]
    h1 = silu(z1)
    z2 = q(h1) @ q(p["W2"]) + p["b2"]
    h2 = silu(z2)
    e = h2 @ p["w3"] + p["b3"][0]
    return e, (z1, h1, z2, h2)


def loss_and_grads(G, atoms_per_config, target, p, emulate_bf16=True):
    """Mean squared error of configuration energies and its gradients (straight through
    the bf16 rounding of the forward operands)."""
    q = (lambda x: bf16(x)) if emulate_bf16 else (lambda x: x)
    e, (z1, h1, z2, h2) = forward(G, p, emulate_bf16)
    C = len(target)
    Es = e.reshape(C, atoms_per_config).sum(axis=1)
    r = Es - target
    loss = float((r ** 2).mean())
    de = np.repeat(2.0 * r / C, atoms_per_config)          # dL/de per row
    g = {"w3": h2.T @ de, "b3": np.array([de.sum()])}
    d2 = np.outer(de, p["w3"]) * dsilu(z2)                  # dL/dz2
    g["W2"] = q(h1).T @ d2
    g["b2"] = d2.sum(axis=0)
    d1 = (d2 @ q(p["W2"]).T) * dsilu(z1)                    # dL/dz1
    g["W1"] = q(G).T @ d1
    g["b1"] = d1.sum(axis=0)
    return loss, g


def adam_step(p, g, state, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
    state["t"] = state.get("t", 0) + 1
    t = state["t"]
    for k in p:
        m = state.setdefault("m_" + k, np.zeros_like(p[k]))
        v = state.setdefault("v_" + k, np.zeros_like(p[k]))
        m[:] = beta1 * m + (1 - beta1) * g[k]
        v[:] = beta2 * v + (1 - beta2) * g[k] ** 2
        mh = m / (1 - beta1 ** t)
        vh = v / (1 - beta2 ** t)
        p[k] = p[k] - lr * mh / (np.sqrt(vh) + eps)
    return p

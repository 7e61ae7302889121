"""CPU oracle of the preconditioner MLP (forward, one-step model loss and its
gradient).  TEST INFRASTRUCTURE ONLY.

Mirrors the arithmetic the kernels are specified to do: BF16 weights, BF16
stored activations after each GELU, FP64 accumulation here (FP32 on the
device), GELU in the tanh form, softplus output.
"""
import numpy as np

H = 64
SIZES = ((3, 64), (64, 64), (64, 64), (64, 1))


def bf16(x):
  """Round-to-nearest-even to bfloat16, returned as float64."""
  a = np.asarray(x, dtype=np.float32)
  u = a.view(np.uint32).astype(np.uint64)
  rounding = ((u >> 16) & 1) + 0x7FFF
  r = ((u + rounding) >> 16) << 16
  return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w):
  w = np.asarray(w, dtype=np.float64)
  out, o = [], 0
  for din, dout in SIZES:
    W = w[o:o + din * dout].reshape(dout, din)
    o += din * dout
    b = w[o:o + dout]
    o += dout
    out.append((W, b))
  return out


def gelu(x):
  return 0.5 * x * (1 + np.tanh(0.7978845608028654 * (x + 0.044715 * x**3)))


def gelu_grad(x):
  u = 0.7978845608028654 * (x + 0.044715 * x**3)
  t = np.tanh(u)
  du = 0.7978845608028654 * (1 + 3 * 0.044715 * x * x)
  return 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * du


def softplus(x):
  return np.where(x > 20, x, np.log1p(np.exp(np.minimum(x, 20))))


def forward(w32, x):
  layers = unpack(w32)
  zs, hs = [], [np.asarray(x, dtype=np.float64)]
  h = hs[0]
  for i, (W, b) in enumerate(layers[:3]):
    z = h @ bf16(W).T + b
    h = bf16(gelu(z))
    zs.append(z)
    hs.append(h)
  W4, b4 = layers[3]
  z4 = h @ bf16(W4).T[:, 0] + b4[0]
  return softplus(z4), (zs, hs, z4)


def loss_and_grad(w32, x, a, c, wt=None):
  """sum wt (s a + s^2 c / 2) and the gradient of its mean."""
  n = x.shape[0]
  wt = np.ones(n) if wt is None else np.asarray(wt, dtype=np.float64)
  s, (zs, hs, z4) = forward(w32, x)
  loss = np.sum(wt * (s * a + 0.5 * s * s * c))
  dz = wt * (a + s * c) / (1 + np.exp(-z4)) / n       # d mean / d z4
  layers = unpack(w32)
  grads = [None] * 4
  W4, _ = layers[3]
  grads[3] = (dz[:, None] * hs[3]).sum(0)[None, :], np.array([dz.sum()])
  d = dz[:, None] * bf16(W4)                          # dH3
  for i in (2, 1, 0):
    W, _ = layers[i]
    dzi = d * gelu_grad(zs[i])
    grads[i] = dzi.T @ hs[i], dzi.sum(0)
    d = dzi @ bf16(W)
  flat = np.concatenate([np.concatenate([g[0].reshape(-1), g[1]]) for g in grads])
  return loss, flat

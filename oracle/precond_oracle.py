"""FP64 numpy restatement of the learned preconditioner's network, loss and
weight gradients.  TEST INFRASTRUCTURE ONLY: the GPU training and inference
kernels (amps_gb300/csrc/precond.cu, precond_tc.cu) are checked against it.

The network has no counterpart in the reference (its GMRES takes only
PrecondParam 0/1, src/pic/pic_field_solver_ecsim.cpp:6232); what is restated
here is the layout and arithmetic the library documents in include/amps_gpu.h:

  x[s][v][3] on the 10^3 region R (v = (k*10 + j)*10 + i, block corner
  (i-1, j-1, k-1)); h1 = conv(x, w1) on R, h2 = conv(h1, w2) on R,
  y = conv(h2, w3) on the owned 8^3 corners (zero padding outside R, no
  activation); z = x + y; loss = mean over owned corners and channels of
  (z - e)^2 with e[s][q][3], q = i + 8j + 64k.
  Weights w[t][cin][cout], tap t = (dx+1) + 3(dy+1) + 9(dz+1).
"""
import numpy as np

TAPS = [(t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1) for t in range(27)]


def _grid(a, ch):
    return np.asarray(a, np.float64).reshape(-1, 10, 10, 10, ch)


def conv(inp, W):
    """out[s,z,y,x,o] = sum_t sum_c W[t,c,o] inp[s,z+dz,y+dy,x+dx,c] (zero outside)"""
    S = inp.shape[0]
    pad = np.zeros((S, 12, 12, 12, inp.shape[-1]))
    pad[:, 1:11, 1:11, 1:11] = inp
    out = np.zeros((S, 10, 10, 10, W.shape[2]))
    for t, (dx, dy, dz) in enumerate(TAPS):
        out += pad[:, 1 + dz:11 + dz, 1 + dy:11 + dy, 1 + dx:11 + dx] @ W[t]
    return out


def owned_mask():
    m = np.zeros((10, 10, 10, 1))
    m[1:9, 1:9, 1:9] = 1.0
    return m


def forward(x, w1, w2, w3):
    """x (S,1000,3) -> (h1, h2, y) on R (y zero off the owned corners)"""
    X = _grid(x, 3)
    h1 = conv(X, np.asarray(w1, np.float64))
    h2 = conv(h1, np.asarray(w2, np.float64))
    y = conv(h2, np.asarray(w3, np.float64)) * owned_mask()
    return X, h1, h2, y


def owned(a):
    """R-grid (S,10,10,10,3) -> (S,512,3) in the owned-corner order"""
    return a[:, 1:9, 1:9, 1:9].reshape(a.shape[0], 512, 3)


def wgrad(dout, inp):
    """dW[t,c,o] = sum dout[s,v,o] inp[s,v+off_t,c]"""
    S = inp.shape[0]
    pad = np.zeros((S, 12, 12, 12, inp.shape[-1]))
    pad[:, 1:11, 1:11, 1:11] = inp
    g = np.zeros((27, inp.shape[-1], dout.shape[-1]))
    for t, (dx, dy, dz) in enumerate(TAPS):
        sh = pad[:, 1 + dz:11 + dz, 1 + dy:11 + dy, 1 + dx:11 + dx]
        g[t] = np.einsum("szyxc,szyxo->co", sh, dout)
    return g


def dgrad(dout, W):
    """din[s,u,c] = sum_t sum_o W[t,c,o] dout[s,u-off_t,o]"""
    S = dout.shape[0]
    pad = np.zeros((S, 12, 12, 12, dout.shape[-1]))
    pad[:, 1:11, 1:11, 1:11] = dout
    din = np.zeros((S, 10, 10, 10, W.shape[1]))
    for t, (dx, dy, dz) in enumerate(TAPS):
        din += pad[:, 1 - dz:11 - dz, 1 - dy:11 - dy, 1 - dx:11 - dx] @ W[t].T
    return din


def loss_grad(x, e, w1, w2, w3):
    """loss and (g1, g2, g3) of the documented objective"""
    w1, w2, w3 = (np.asarray(w, np.float64) for w in (w1, w2, w3))
    X, h1, h2, y = forward(x, w1, w2, w3)
    S = X.shape[0]
    E = np.zeros_like(y)
    E[:, 1:9, 1:9, 1:9] = np.asarray(e, np.float64).reshape(S, 8, 8, 8, 3)
    r = (X + y - E) * owned_mask()
    n = S * 512 * 3
    loss = float(np.sum(r * r) / n)
    dy = 2.0 * r / n
    g3 = wgrad(dy, h2)
    dh2 = dgrad(dy, w3)
    g2 = wgrad(dh2, h1)
    dh1 = dgrad(dh2, w2)
    g1 = wgrad(dh1, X)
    return loss, (g1, g2, g3)

"""FP64 CPU restatement of the learned prober's loss and gradient (test
infrastructure only; checks the library's CUDA forward/backward kernels).

Network (per example b, candidates i = 0..63 with list ids c and features f):
    h1 = relu(b1 + sum_i f_i W1[c_i]);  h2 = relu(W2 h1 + b2)
    z_i = W3[c_i] . h2 + b3[c_i];       loss = sum_{b,i valid} BCE(z_i, y_i) / (B * 64)
Candidates with id -1 contribute nothing.
"""
import numpy as np


def loss_grad(W1, b1, W2, b2, W3, b3, cand, feat, lab):
    W1, b1, W2, b2, W3, b3 = (np.asarray(a, np.float64) for a in (W1, b1, W2, b2, W3, b3))
    cand = np.asarray(cand)
    feat = np.asarray(feat, np.float64)
    lab = np.asarray(lab, np.float64)
    B, C = cand.shape
    valid = cand >= 0
    cc = np.where(valid, cand, 0)
    fw = np.where(valid, feat, 0.0)
    h1p = b1 + np.einsum("bi,bih->bh", fw, W1[cc])
    h1 = np.maximum(h1p, 0)
    h2p = h1 @ W2.T + b2
    h2 = np.maximum(h2p, 0)
    z = np.einsum("bih,bh->bi", W3[cc], h2) + b3[cc]
    norm = 1.0 / (B * C)
    bce = np.maximum(z, 0) - lab * z + np.log1p(np.exp(-np.abs(z)))
    loss = float((bce * valid).sum() * norm)
    dz = (1 / (1 + np.exp(-z)) - lab) * norm * valid
    gW3 = np.zeros_like(W3)
    gb3 = np.zeros_like(b3)
    np.add.at(gW3, cc[valid], (dz[:, :, None] * h2[:, None, :])[valid])
    np.add.at(gb3, cc[valid], dz[valid])
    dh2 = np.einsum("bi,bih->bh", dz, W3[cc]) * (h2p > 0)
    gW2 = dh2.T @ h1
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ W2) * (h1p > 0)
    gb1 = dh1.sum(0)
    gW1 = np.zeros_like(W1)
    np.add.at(gW1, cc[valid], (fw[:, :, None] * dh1[:, None, :])[valid])
    return loss, (gW1, gb1, gW2, gb2, gW3, gb3)

"""numpy restatement of the deformed-box geometric factors
(nekbone_gb300/csrc/nb_geom.cu) for the tests: trilinear elements whose
vertices are displaced by amp*h*sum_q a_q sin(k_q.X + phi_q), G = w |J| J^-1
J^-T at the GLL points."""
from __future__ import annotations

import math

import numpy as np

M64 = (1 << 64) - 1


def _splitmix64(state):
    state[0] = (state[0] + 0x9E3779B97F4A7C15) & M64
    z = state[0]
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def modes(seed, nelx, nely, nelz):
    s = [seed & M64]
    L = (2.0 * nelx, 2.0 * nely, 2.0 * nelz)
    twopi = 8.0 * math.atan(1.0)
    a, k, phi = np.zeros((4, 3)), np.zeros((4, 3)), np.zeros(4)
    for q in range(4):
        for d in range(3):
            a[q, d] = 2.0 * ((_splitmix64(s) >> 11) / 9007199254740992.0) - 1.0
        for d in range(3):
            k[q, d] = twopi * (1 + _splitmix64(s) % 3) / L[d]
        phi[q] = twopi * ((_splitmix64(s) >> 11) / 9007199254740992.0)
    return a, k, phi


def deformed_g(nelx, nely, nelz, z, w, seed, amp=0.1):
    a, kk, phi = modes(seed, nelx, nely, nelz)
    lx = len(z)
    out = np.zeros((nelz, nely, nelx, lx, lx, lx, 6))
    R, S, T = np.meshgrid(z, z, z, indexing="ij")  # R[i,j,k] = z[i]
    W = w[:, None, None] * w[None, :, None] * w[None, None, :]
    for ez in range(nelz):
        for ey in range(nely):
            for ex in range(nelx):
                X = np.zeros((8, 3))
                for v in range(8):
                    P = np.array([2.0 * (ex + (v & 1)), 2.0 * (ey + ((v >> 1) & 1)),
                                  2.0 * (ez + ((v >> 2) & 1))])
                    d = np.zeros(3)
                    for q in range(4):
                        d += a[q] * math.sin(kk[q] @ P + phi[q])
                    X[v] = P + amp * 2.0 * d
                J = np.zeros((3, 3) + R.shape)
                for v in range(8):
                    sr = 1.0 if v & 1 else -1.0
                    ss = 1.0 if (v >> 1) & 1 else -1.0
                    st = 1.0 if (v >> 2) & 1 else -1.0
                    fr, fs, ft = 0.5 * (1 + sr * R), 0.5 * (1 + ss * S), 0.5 * (1 + st * T)
                    for ax in range(3):
                        J[ax, 0] += 0.5 * sr * fs * ft * X[v, ax]
                        J[ax, 1] += 0.5 * ss * fr * ft * X[v, ax]
                        J[ax, 2] += 0.5 * st * fr * fs * X[v, ax]
                Jm = np.moveaxis(J, (0, 1), (-2, -1))        # (...,3,3)
                det = np.linalg.det(Jm)
                Ji = np.linalg.inv(Jm)
                G = (W * det)[..., None, None] * (Ji @ np.swapaxes(Ji, -1, -2))
                gg = np.stack([G[..., 0, 0], G[..., 0, 1], G[..., 0, 2],
                               G[..., 1, 1], G[..., 1, 2], G[..., 2, 2]], axis=-1)
                # element layout (i fastest): index [k, j, i]
                out[ez, ey, ex] = np.transpose(gg, (2, 1, 0, 3))
    return out.reshape(-1)

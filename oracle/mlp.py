"""CPU restatement of the constraint warm-start network (test infrastructure:
only the tests load it).

Restates, in numpy, what the device computes for the SHAKE warm start: the 12
per-constraint features (the same FP64 operations in the same order, rounded
once to FP32), the 12-64-64-1 SiLU network with its matmul weights and
activations rounded to BF16, and the gradient of the mean squared error with
the roundings treated as the identity.  Sums here are FP64, so device results
(FP32 sums) agree to FP32 accuracy; a BF16 rounding that lands on the other
side of a tie moves one activation by one BF16 step, rarely.

The multiplier being predicted is the sum of the Jacobi lambdas of
constraint::solve (geodesic-engine/src/constraint.rs:62-152), made
dimensionless as t = Lambda * 2 (1/m_i + 1/m_j); the network's output is the
standardised correction t - t1 to the first Jacobi step t1.
"""
import numpy as np

N_IN, N_H = 12, 64
OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3, OFF_B3, NPAR = 0, 768, 832, 4928, 4992, 5056, 5057


def bf16(x):
    """Round float32 values to BF16 (nearest, ties to even), as float32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def unpack(P):
    P = np.asarray(P)
    if P.dtype != np.float64:
        P = P.astype(np.float32)
    return (P[OFF_W1:OFF_B1].reshape(N_IN, N_H), P[OFF_B1:OFF_W2], P[OFF_W2:OFF_B2].reshape(N_H, N_H),
            P[OFF_B2:OFF_W3], P[OFF_W3:OFF_B3], P[OFF_B3])


def features(constr_i, constr_j, dsq, pos, ref, inv_mass):
    """Raw features [C][12] (float32), scale 2 (1/m_i + 1/m_j) [C] and the
    first Jacobi step t1 = (|d|^2 - d0^2) / (d . r) [C] (constraint.rs:110-115
    times the scale), with r = ref_i - ref_j, d = pos_i - pos_j:

      0 (d.d - d0^2)/d0^2   1 d.r/d0^2   2 d0   3 1/m_i   4 1/m_j
      5, 6 constraints on i, on j   7 t1
      8 c1 = sum over the other constraints l on a shared atom a of
            (1/m_a)/w_k cos(r_k, r_l) s_k s_l t1_l w_k/w_l
      9 sum of the squared coupling coefficients   10 max |cos|   11 sum t1_l

    (s = +1 where a is the constraint's i, -1 where it is its j; w = 1/m_i +
    1/m_j.)  FP64 only where it cancels: the coordinate differences,
    |d|^2 - d0^2 and d . r, each rounded once to FP32; the ratios, t1 and d0
    are correctly rounded FP32 operations.  Features 8-11 in FP32 (masses, t1
    and the FP64 bond vectors rounded to FP32 first), in the device's order:
    atom i's constraints, then atom j's, each ascending."""
    ci = [int(v) for v in constr_i]
    cj = [int(v) for v in constr_j]
    dsq = [float(v) for v in dsq]
    inv = [float(v) for v in inv_mass]
    C = len(ci)
    rows = {}
    for k in range(C):
        rows.setdefault(ci[k], []).append((k, 1.0))
        rows.setdefault(cj[k], []).append((k, -1.0))
    X, Y, Z = [list(map(float, pos[d])) for d in range(3)]
    RX, RY, RZ = [list(map(float, ref[d])) for d in range(3)]

    def dot3(ax, ay, az, bx, by, bz):
        return (ax * bx + ay * by) + az * bz

    f32 = np.float32

    def unit(k):
        # FP32: the FP64 difference rounded once, then float32 operations
        i, j = ci[k], cj[k]
        rx, ry, rz = f32(RX[i] - RX[j]), f32(RY[i] - RY[j]), f32(RZ[i] - RZ[j])
        il = f32(1.0) / np.sqrt(dot3(rx, ry, rz, rx, ry, rz))
        return rx * il, ry * il, rz * il

    f = np.empty((C, N_IN), np.float32)
    t1 = np.zeros(C)
    scale = np.zeros(C)
    for k in range(C):
        i, j = ci[k], cj[k]
        rx, ry, rz = RX[i] - RX[j], RY[i] - RY[j], RZ[i] - RZ[j]
        tx, ty, tz = X[i] - X[j], Y[i] - Y[j], Z[i] - Z[j]
        num = f32(dot3(tx, ty, tz, tx, ty, tz) - dsq[k])
        dr = f32(dot3(tx, ty, tz, rx, ry, rz))
        d0f = f32(dsq[k])
        t1f = f32(0.0) if dr == 0.0 else num / dr
        t1[k] = float(t1f)
        scale[k] = 2.0 * (inv[i] + inv[j])
        f[k, :8] = [num / d0f, dr / d0f, np.sqrt(d0f), inv[i], inv[j], len(rows[i]), len(rows[j]), t1f]
    for k in range(C):
        wk = f32(inv[ci[k]]) + f32(inv[cj[k]])
        ux, uy, uz = unit(k)
        c1 = c2 = cmax = ct = f32(0.0)
        for at, sk in ((ci[k], f32(1.0)), (cj[k], f32(-1.0))):
            ia = f32(inv[at])
            for l, sl in rows[at]:
                if l == k:
                    continue
                vx, vy, vz = unit(l)
                cs = dot3(ux, uy, uz, vx, vy, vz)
                wl = f32(inv[ci[l]]) + f32(inv[cj[l]])
                coup = ((ia / wk) * cs) * (sk * f32(sl))
                tl = f32(t1[l])
                c1 = c1 + ((coup * tl) * wk) / wl
                c2 = c2 + coup * coup
                cmax = max(cmax, abs(cs))
                ct = ct + tl
        f[k, 8:] = [c1, c2, cmax, ct]
    return f, scale, t1


def standardize(f, norm):
    norm = np.asarray(norm, np.float32)
    return (np.asarray(f, np.float32) - norm[:N_IN]) / norm[N_IN:2 * N_IN]


def _silu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return z * s, s * (1.0 + z * (1.0 - s))


def forward(P, x, emulate_bf16=True):
    """Outputs y [m] for standardised inputs x [m][12]; also the cache the
    backward pass needs."""
    W1, b1, W2, b2, w3, b3 = unpack(P)
    rd = bf16 if emulate_bf16 else (lambda v: np.asarray(v, np.float64))
    xb = rd(x).astype(np.float64)
    z1 = b1.astype(np.float64) + xb @ rd(W1).astype(np.float64)
    a1, d1 = _silu(z1)
    a1b = rd(a1.astype(np.float32) if emulate_bf16 else a1).astype(np.float64)
    z2 = b2.astype(np.float64) + a1b @ rd(W2).astype(np.float64)
    a2, d2 = _silu(z2)
    a2b = rd(a2.astype(np.float32) if emulate_bf16 else a2).astype(np.float64)
    y = float(b3) + a2b @ rd(w3).astype(np.float64)
    return y, (xb, a1b, a2b, d1, d2, rd(W2).astype(np.float64), rd(w3).astype(np.float64))


def gradient(P, x, t, emulate_bf16=True):
    """Gradient [5057] of mean((y - t)^2) and the loss (FP64)."""
    y, (xb, a1b, a2b, d1, d2, W2, w3) = forward(P, x, emulate_bf16)
    m = len(t)
    r = y - np.asarray(t, np.float64)
    dy = 2.0 * r / m
    g = np.zeros(NPAR)
    g[OFF_W3:OFF_B3] = a2b.T @ dy
    g[OFF_B3] = dy.sum()
    dz2 = (dy[:, None] * w3[None, :]) * d2
    g[OFF_W2:OFF_B2] = (a1b.T @ dz2).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz1 = (dz2 @ W2.T) * d1
    g[OFF_W1:OFF_B1] = (xb.T @ dz1).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    return g, float(np.mean(r * r))


def glorot(seed):
    """Random parameters for tests (not the device's initialiser)."""
    rng = np.random.default_rng(seed)
    P = np.zeros(NPAR, np.float32)
    for off, fi, fo in ((OFF_W1, N_IN, N_H), (OFF_W2, N_H, N_H), (OFF_W3, N_H, 1)):
        a = np.sqrt(6.0 / (fi + fo))
        P[off:off + fi * fo] = rng.uniform(-a, a, fi * fo)
    P[OFF_B1:OFF_W2] = rng.normal(0, 0.1, N_H)
    P[OFF_B2:OFF_W3] = rng.normal(0, 0.1, N_H)
    P[OFF_B3] = 0.05
    return P

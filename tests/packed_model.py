"""numpy model of the GPU algorithm (lenslet-grid transfer matrices, packed layout).

Mirrors, index for index, what libflf.so computes: the lenslet-grid kernels
K_iq built from the stored PSF quadrant (k_build_k), their f x f spectra,
the packed [freq pair][row][slot] layout with zeroed duplicates (k_pack), and
the symmetric multiply-accumulate (k_mac).  Tests compare it with the oracle
so that the mathematics of the kernels is checked on the CPU.
"""

import numpy as np


def smooth_even_at_least(n):
    f = max(n, 2)
    while True:
        if f % 2 == 0:
            m = f
            for p in (2, 3, 5, 7):
                while m % p == 0:
                    m //= p
            if m == 1:
                return f
        f += 1


def kernel_radius(h, N):
    return ((h - 1) // 2 + N - 1) // N


def choose_f(Y, X, hs, N):
    Ly, Lx = -(-Y // N), -(-X // N)
    R = max(kernel_radius(h, N) for h in hs)
    return smooth_even_at_least(max(max(Ly, Lx) + R, 2 * R + 1))


def hfull_value(Hred, N, b, a, y, x):
    """Value of the expanded PSF Hfull[b][a][y, x] via the reference's symmetry map."""
    c = N // 2
    h = Hred.shape[-1]
    bb, aa = min(b, N - 1 - b), min(a, N - 1 - a)
    yy = h - 1 - y if b > c else y
    xx = h - 1 - x if a > c else x
    return Hred[bb, aa, yy, xx] if aa >= bb else Hred[aa, bb, xx, yy]


def kernel_image(Hred, N, i, q, f):
    h = Hred.shape[-1]
    ch = (h - 1) // 2
    R = kernel_radius(h, N)
    b, a = divmod(i, N)
    be, al = divmod(q, N)
    K = np.zeros((f, f))
    for m in range(-R, R + 1):
        y = m * N + be - b + ch
        if y < 0 or y >= h:
            continue
        for n in range(-R, R + 1):
            x = n * N + al - a + ch
            if 0 <= x < h:
                K[m % f, n % f] = hfull_value(Hred, N, b, a, y, x)
    return K


def tables(N):
    c = N // 2
    NN = N * N
    My = lambda i: (N - 1 - i // N) * N + i % N  # noqa: E731
    Mx = lambda i: (i // N) * N + (N - 1 - i % N)  # noqa: E731
    Mxy = lambda i: NN - 1 - i  # noqa: E731
    slotcol, okind = [], []
    for be in range(c):
        for al in range(c):
            q = be * N + al
            slotcol += [q, My(q), Mx(q), Mxy(q)]
            okind.append(0)
    for be in range(c):
        q = be * N + c
        slotcol += [q, My(q)]
        okind.append(1)
    for al in range(c):
        q = c * N + al
        slotcol += [q, Mx(q)]
        okind.append(2)
    slotcol.append(c * N + c)
    okind.append(3)
    reps = []   # (channel, kind, first row)
    row = 0
    for b in range(c):
        for a in range(N):
            if a != c:
                reps.append((b * N + a, 0, row))
                row += 1
    for k in range(2 * c + 1):
        if k < c:
            reps.append((k * N + c, 1, row))
        elif k < 2 * c:
            reps.append((c * N + (k - c), 2, row))
        else:
            reps.append((c * N + c, 3, row))
        row += 2
    return dict(slotcol=slotcol, okind=okind, reps=reps, nrow=row, My=My, Mx=Mx, Mxy=Mxy, c=c)


def packed_matrices(Hred, N, f):
    """P[kpair, row, slot] for one plane: the layout k_pack writes (scaled by 1/f^2)."""
    tb = tables(N)
    NN = N * N
    fq = f // 2 + 1
    P = np.zeros((fq * fq, tb["nrow"], NN), np.complex128)
    colslot = np.empty(NN, int)
    colslot[tb["slotcol"]] = np.arange(NN)
    for ch, kind, row in tb["reps"]:
        spec = np.stack([np.fft.rfft2(kernel_image(Hred, N, ch, q, f)) for q in range(NN)]) / (f * f)
        for uy in range(fq):
            us = (-uy) % f
            for ux in range(fq):
                kp = uy * fq + ux
                selfp = us == uy
                if kind == 0:
                    if not (selfp and ch % N > N // 2):
                        P[kp, row, colslot] = spec[:, uy, ux]
                else:
                    P[kp, row, colslot] = spec[:, uy, ux]
                    if not selfp:
                        P[kp, row + 1, colslot] = spec[:, us, ux]
    return P


SIG = {0: dict(y=[1, 0, 3, 2], x=[2, 3, 0, 1], xy=[3, 2, 1, 0]),
       1: dict(y=[1, 0], x=[0, 1], xy=[1, 0]),
       2: dict(y=[0, 1], x=[1, 0], xy=[1, 0]),
       3: dict(y=[0], x=[0], xy=[0])}


def packed_mac(Ps, Ss, N, f):
    """out[j, uy, ux] = sum over planes of T_z S_z, evaluated from packed matrices."""
    tb = tables(N)
    NN = N * N
    fq = f // 2 + 1
    My, Mx, Mxy = tb["My"], tb["Mx"], tb["Mxy"]
    out = np.zeros((NN, f, fq), np.complex128)
    for uy in range(fq):
        us = (-uy) % f
        for ux in range(fq):
            kp = uy * fq + ux
            s0 = 0
            accs = []
            for ok in tb["okind"]:
                ns = {0: 4, 1: 2, 2: 2, 3: 1}[ok]
                accs.append((s0, ns, ok, np.zeros(ns, complex), np.zeros(ns, complex)))
                s0 += ns
            for P, S in zip(Ps, Ss):
                Su, Ss_ = S[:, uy, ux], S[:, us, ux]
                for ch, kind, row in tb["reps"]:
                    for s0, ns, ok, U, V in accs:
                        sg = SIG[ok]
                        t = P[kp, row, s0:s0 + ns]
                        if kind == 0:
                            sv = (Su[ch], Su[Mxy(ch)], Ss_[My(ch)], Ss_[Mx(ch)])
                            for k in range(ns):
                                U[k] += t[k] * sv[0] + np.conj(t[sg["xy"][k]]) * sv[1]
                                V[sg["y"][k]] += t[k] * sv[2]
                                V[sg["x"][k]] += np.conj(t[k]) * sv[3]
                        else:
                            s = P[kp, row + 1, s0:s0 + ns]
                            M = My if kind == 1 else Mx
                            sv = (Su[ch], Ss_[ch], Ss_[M(ch)], Su[M(ch)])
                            for k in range(ns):
                                U[k] += t[k] * sv[0]
                                V[k] += s[k] * sv[1]
                                if kind == 1:
                                    V[sg["y"][k]] += t[k] * sv[2]
                                    U[sg["y"][k]] += s[k] * sv[3]
                                elif kind == 2:
                                    V[sg["x"][k]] += np.conj(t[k]) * sv[2]
                                    U[sg["x"][k]] += np.conj(s[k]) * sv[3]
            for s0, ns, ok, U, V in accs:
                for k in range(ns):
                    q = tb["slotcol"][s0 + k]
                    if us == uy:
                        out[q, uy, ux] = U[k] + V[k]
                    else:
                        out[q, uy, ux] = U[k]
                        out[q, us, ux] = V[k]
    return out


def channel_spectra(img, N, f):
    Y, X = img.shape
    S = np.zeros((N * N, f, f // 2 + 1), complex)
    for i in range(N * N):
        b, a = divmod(i, N)
        s = np.zeros((f, f))
        sub = img[b::N, a::N]
        s[:sub.shape[0], :sub.shape[1]] = sub
        S[i] = np.fft.rfft2(s)
    return S


def to_pixels(out, N, f, Y, X):
    img = np.zeros((Y, X))
    for j in range(N * N):
        be, al = divmod(j, N)
        r = np.fft.irfft2(out[j], s=(f, f)) * (f * f)
        sub = img[be::N, al::N]
        sub[:] = r[:sub.shape[0], :sub.shape[1]]
    return img


def forward_model(H_planes, vol, N):
    """Forward projection of vol [Z, Y, X] through the packed algorithm."""
    Z, Y, X = vol.shape
    f = choose_f(Y, X, [h.shape[-1] for h in H_planes], N)
    Ps = [packed_matrices(np.asarray(h, np.float64), N, f) for h in H_planes]
    Ss = [channel_spectra(vol[z], N, f) for z in range(Z)]
    return to_pixels(packed_mac(Ps, Ss, N, f), N, f, Y, X)


def backward_model(Ht_planes, img, N):
    Y, X = img.shape
    f = choose_f(Y, X, [h.shape[-1] for h in Ht_planes], N)
    S = channel_spectra(img, N, f)
    out = []
    for h in Ht_planes:
        P = packed_matrices(np.asarray(h, np.float64), N, f)
        out.append(to_pixels(packed_mac([P], [S], N, f), N, f, Y, X))
    return np.stack(out)

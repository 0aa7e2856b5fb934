"""numpy model of the GPU algorithm (lenslet-grid transfer matrices, packed layout).

Mirrors, index for index, what libflf.so computes: the lenslet-grid kernels
K_iq built from the stored PSF quadrant (k_build_k), their f x f spectra,
the packed [frequency quad][row][slot] layout (k_pack), and the symmetric
multiply-accumulate that uses the mirror and transpose symmetries (k_mac).  Tests compare it with the oracle
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
    """Index tables of the packed layout.

    Output side (slots of a stored row): the mirror orbits of output channels,
    slot-major as in the kernel.  Input side (stored rows of one half block):
    the generic orbits (b, a'), a' <= b < c, as their two rows i = (b, a') and
    Mx i = (b, N-1-a'); then the centre-cross representatives (b, c), b < c,
    and the centre (c, c) as row pairs (u, u*).  Orbits with a' < b (stored
    first) and the (b, c) pairs are transposable: their transposes (a', b) and
    (c, b) get no rows of their own."""
    c = N // 2
    NN = N * N
    My = lambda i: (N - 1 - i // N) * N + i % N  # noqa: E731
    Mx = lambda i: (i // N) * N + (N - 1 - i % N)  # noqa: E731
    Mxy = lambda i: NN - 1 - i  # noqa: E731
    Tr = lambda i: (i % N) * N + i // N  # noqa: E731
    slotcol, okind, offs = [], [], []
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
    colslot = np.empty(NN, int)
    colslot[slotcol] = np.arange(NN)
    # virtual slots [q, My q, Mx q, Mxy q] of every output orbit (degenerate orbits repeat)
    s0 = 0
    for ok in okind:
        if ok == 0:
            off = [s0, s0 + 1, s0 + 2, s0 + 3]
        elif ok == 1:
            off = [s0, s0 + 1, s0, s0 + 1]
        elif ok == 2:
            off = [s0, s0, s0 + 1, s0 + 1]
        else:
            off = [s0] * 4
        ns = {0: 4, 1: 2, 2: 2, 3: 1}[ok]
        offT = [int(colslot[Tr(slotcol[o])]) for o in off]
        offs.append((off, offT, ns, ok))
        s0 += ns
    groups = []     # (channel, kind, first row, transposable, mx_row)
    row = 0
    orbits = [(b, ap) for b in range(c) for ap in range(b)] + [(b, b) for b in range(c)]
    for b, ap in orbits:
        for a in (ap, N - 1 - ap):
            groups.append((b * N + a, 0, row, ap < b, a > c))
            row += 1
    for b in range(c):
        groups.append((b * N + c, 1, row, True, False))
        row += 2
    groups.append((c * N + c, 3, row, False, False))
    row += 2
    return dict(slotcol=slotcol, colslot=colslot, okind=okind, offs=offs, groups=groups, nrow=row,
                My=My, Mx=Mx, Mxy=Mxy, Tr=Tr, c=c)


def quads(fq):
    """Frequency quads in kernel order: k -> (uy, ux), uy <= ux, ux-major; and the
    first stored row of each (in half blocks: a diagonal quad holds one)."""
    out = []
    for ux in range(fq):
        for uy in range(ux + 1):
            k = len(out)
            out.append((uy, ux, 2 * k - ux))
    return out


def packed_matrices(Hred, N, f):
    """P[half block, row, slot] for one plane: the layout k_pack writes (scaled by 1/f^2).

    Quad (uy, ux), uy < ux, holds two half blocks: rows of frequency pair
    (uy, ux) then rows of (ux, uy); a diagonal quad (uy = ux) holds one.  The
    second half block keeps its columns in transposed order (the slot of output
    channel j holds channel Tr j), so that both sides of a quad read every half
    block at their own slots."""
    tb = tables(N)
    NN = N * N
    fq = f // 2 + 1
    P = np.zeros((fq * fq, tb["nrow"], NN), np.complex128)
    colslot = tb["colslot"]
    colslotT = colslot[[tb["Tr"](q) for q in range(NN)]]
    for ch, kind, row, _, _ in tb["groups"]:
        spec = np.stack([np.fft.rfft2(kernel_image(Hred, N, ch, q, f)) for q in range(NN)]) / (f * f)
        for uy, ux, hb in quads(fq):
            for side, (py, px) in enumerate(((uy, ux), (ux, uy))):
                if side == 1 and uy == ux:
                    continue
                ps = (-py) % f
                cs = colslotT if side else colslot
                P[hb + side, row, cs] = spec[:, py, px]
                if kind != 0:
                    P[hb + side, row + 1, cs] = spec[:, ps, px]
    return P


SIG = dict(y=[1, 0, 3, 2], x=[2, 3, 0, 1], xy=[3, 2, 1, 0])


def _operands(tb, ch, kind, mxrow, use, recv_self):
    """Input channels (with the frequency: 0 = u, 1 = u*) and conjugation of the
    four operand pairs of a row group, for its own side (use 0) or the other side
    of the quad through the transpose (use 1); zero operands where the receiving
    frequency pair is self-paired and the term would count twice."""
    My, Mx, Mxy, Tr = tb["My"], tb["Mx"], tb["Mxy"], tb["Tr"]
    if use == 1:
        ch = Tr(ch)
    if kind == 0:
        ops = [(ch, 0, False), (Mxy(ch), 0, True), (My(ch), 1, False), (Mx(ch), 1, True)]
        zero = [mxrow and recv_self] * 4
    elif kind == 1 and use == 0:
        ops = [(ch, 0, False), (ch, 1, False), (My(ch), 1, False), (My(ch), 0, False)]
        zero = [False, recv_self, False, recv_self]
    elif kind == 1:     # transposed (b, c) row pair: a (c, b) channel, conjugated u* terms
        ops = [(ch, 0, False), (ch, 1, True), (Mx(ch), 1, True), (Mx(ch), 0, False)]
        zero = [False, recv_self, False, recv_self]
    else:
        ops = [(ch, 0, False), (ch, 1, False), (ch, 0, False), (ch, 0, False)]
        zero = [False, recv_self, True, True]
    return ops, zero


def packed_mac(Ps, Ss, N, f):
    """out[j, uy, ux] = sum over planes of T_z S_z, evaluated as the kernel does.

    Per quad, side-0 and side-1 threads handle frequency pairs (uy, ux) and
    (ux, uy).  Thread t of side 0 owns output orbit t (virtual slots [q, My q,
    Mx q, Mxy q]); thread t of side 1 owns the transposed orbit, virtual slots
    [Tr q, Tr My q, Tr Mx q, Tr Mxy q] = [r, Mx r, My r, Mxy r] (r = Tr q), so
    its My and Mx slot permutations trade places.  Both read every row at the
    slots of orbit t: a row feeds its own side, and transposable rows also feed
    the other side through the transpose.  A diagonal quad adds side 1 into
    side 0 (thread T(t), My / Mx slots swapped)."""
    tb = tables(N)
    NN = N * N
    fq = f // 2 + 1
    Tr = tb["Tr"]
    out = np.zeros((NN, f, fq), np.complex128)
    swap = [0, 2, 1, 3]
    for uy, ux, hb in quads(fq):
        diag = uy == ux
        freqs = [(uy, ux), (ux, uy)]
        selfp = [(-p[0]) % f == p[0] for p in freqs]
        acc = [[(np.zeros(4, complex), np.zeros(4, complex)) for _ in tb["offs"]] for _ in range(2)]
        for P, S in zip(Ps, Ss):
            comb = [(S[:, p[0], p[1]], S[:, (-p[0]) % f, p[1]]) for p in freqs]
            for bs in range(1 if diag else 2):
                for ch, kind, row, trans, mxrow in tb["groups"]:
                    for ts in range(2):
                        use = 0 if ts == bs else 1
                        if use == 1 and not trans:
                            continue
                        ops, zero = _operands(tb, ch, kind, mxrow, use, selfp[ts])
                        sv = [0 if z else comb[ts][st][ci] for (ci, st, cj), z in zip(ops, zero)]
                        sy = SIG["x"] if ts else SIG["y"]
                        sx = SIG["y"] if ts else SIG["x"]
                        for o, (off, offT, ns, ok) in enumerate(tb["offs"]):
                            U, V = acc[ts][o]
                            t = P[hb + bs, row, off]
                            cj = lambda v, k: np.conj(v) if ops[k][2] else v  # noqa: E731
                            if kind == 0:
                                for k in range(4):
                                    U[k] += cj(t[k], 0) * sv[0] + cj(t[SIG["xy"][k]], 1) * sv[1]
                                    V[sy[k]] += cj(t[k], 2) * sv[2]
                                    V[sx[k]] += cj(t[k], 3) * sv[3]
                            else:
                                s = P[hb + bs, row + 1, off]
                                for k in range(4):
                                    U[k] += cj(t[k], 0) * sv[0]
                                    V[k] += cj(s[k], 1) * sv[1]
                                    if kind == 1 and use == 0:
                                        V[sy[k]] += cj(t[k], 2) * sv[2]
                                        U[sy[k]] += cj(s[k], 3) * sv[3]
                                    elif kind == 1:
                                        V[sx[k]] += cj(t[k], 2) * sv[2]
                                        U[sx[k]] += cj(s[k], 3) * sv[3]
        if diag:
            # side-1 thread t holds the transposed orbit of t, i.e. the orbit of thread T(t)
            for o, (off, offT, ns, ok) in enumerate(tb["offs"]):
                q = tb["slotcol"][off[0]]
                o2 = [i for i, ent in enumerate(tb["offs"]) if tb["slotcol"][ent[0][0]] == Tr(q)][0]
                U1, V1 = acc[1][o]
                U0, V0 = acc[0][o2]
                for k in range(4):
                    U0[swap[k]] += U1[k]
                    V0[swap[k]] += V1[k]
        for ts in range(2):
            if diag and ts == 1:
                break
            py, px = freqs[ts]
            ps = (-py) % f
            for o, (off, offT, ns, ok) in enumerate(tb["offs"]):
                U, V = acc[ts][o]
                for k in range(ns):
                    vk = {0: k, 1: k, 2: 2 * k, 3: 0}[ok]
                    q = tb["slotcol"][off[vk]]
                    if ts:
                        q = Tr(q)
                    if selfp[ts]:
                        out[q, py, px] = U[vk] + V[vk]
                    else:
                        out[q, py, px] = U[vk]
                        out[q, ps, px] = V[vk]
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

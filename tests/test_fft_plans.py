"""The index arithmetic of the kernels' Stockham plans, restated in numpy and checked
against numpy's FFT filter (CPU only; the GPU tests check the kernels themselves).

* fused kernel, compile-time line plans (fused_impl.cuh ct_pass / ct_mid): factors
  8, 8, ..., 4 or 2; intermediate lines in the padded layout padi(i) = i + i / 16,
  addressed as a per-lane base plus compile-time offsets; per-pass twiddle tables
  (clv_launch.h tw_*_off, pass_twiddle_source);
* in-place line filters (inplace_fft.cuh, used by the plane filter of k_plane.cu and
  the strided-axis tiles of k_axis.cu): Cooley-Tukey passes over a tile of lines
  (decimation in frequency forward, the filter at the digit-reversed frequencies,
  decimation in time back), butterfly b = line b % NL, index b / NL, with the thread
  counts of clv_launch.h plane_threads or 256;
* whole lines in registers (k_plane.cu plane_lines_in_registers, k_axis.cu
  axis_line_kernel): the radix-64 butterfly and twiddle tables of fft_radix.cuh, the
  transposition addresses and the tiles' coverage of a slice.
"""
import numpy as np
import pytest


def padi(i):
    return i + (i >> 4)


def p2_plan(n):
    f = []
    while n % 8 == 0:
        f.append(8)
        n //= 8
    while n % 4 == 0:
        f.append(4)
        n //= 4
    while n % 2 == 0:
        f.append(2)
        n //= 2
    return f


def ax_plan(n0):
    """Axis-filter and plane plans: 128 = 16 x 8, else factors 8, 4, 2, 3, 5 in order."""
    f, n = [], n0
    while n > 1:
        r = 16 if (n0 == 128 and n == 128) else next(x for x in (8, 4, 2, 3, 5) if n % x == 0)
        f.append(r)
        n //= r
    return f


def dft(v, S):
    """y_q = sum_r v_r exp(S 2 pi i r q / R) along the last axis (the kernels' Radix<R>)."""
    R = v.shape[-1]
    r = np.arange(R)
    return v @ np.exp(S * 2j * np.pi * np.outer(r, r) / R)


def passes(plan):
    """(R, NS, S, mid) of the forward passes, the middle pass and the inverse passes."""
    out, ns = [], 1
    for r in plan[:-1]:
        out.append((r, ns, -1, False))
        ns *= r
    out.append((plan[-1], ns, -1, True))
    ns = plan[-1]
    for r in reversed(plan[:-1]):
        out.append((r, ns, +1, False))
        ns *= r
    return out


def tw_tables(n):
    """Per-pass twiddle tables of the fused kernel (layout of tw_*_off): pass (R, NS)
    holds w^(k r) at (r - 1) NS + k, conjugated for the inverse passes; the middle
    pass holds w^(j r) at (r - 1) n/R + j."""
    w = np.exp(-2j * np.pi * np.arange(n) / n)
    tabs = []
    for R, NS, S, mid in passes(p2_plan(n)):
        if not mid and NS == 1:
            tabs.append(None)
            continue
        nR = n // R
        span = nR if mid else NS
        tstep = 1 if mid else n // (NS * R)
        t = np.empty((R - 1) * span, complex)
        for r in range(1, R):
            for k in range(span):
                v = w[k * r * tstep]
                t[(r - 1) * span + k] = np.conj(v) if (S > 0 and not mid) else v
        tabs.append(t)
    return tabs


def tw_entries(n):
    return sum(0 if t is None else len(t) for t in tw_tables(n))


def test_pass_table_sizes_match_the_static_asserts():
    # fused_impl.cuh: tw_entries(256) == 500, tw_entries(128) == 246, tw_entries(64) == 112
    assert (tw_entries(256), tw_entries(128), tw_entries(64)) == (500, 246, 112)


@pytest.mark.parametrize("n", [64, 128, 256, 512])
def test_padded_addresses_split_into_lane_base_and_offset(n):
    """ct_pass: padi(j + r nR) = padi(j) + padi(r nR), padi(o + q NS) = padi(o) + padi(q NS);
    ct_mid: padi(j R + q) = padi(j R) + q."""
    for R, NS, S, mid in passes(p2_plan(n)):
        nR = n // R
        for j in range(nR):
            for r in range(R):
                assert padi(j + r * nR) == padi(j) + padi(r * nR)
            if mid:
                for q in range(R):
                    assert padi(j * R + q) == padi(j * R) + q
            else:
                o = (j // NS) * NS * R + j % NS
                for q in range(R):
                    assert padi(o + q * NS) == padi(o) + padi(q * NS)


@pytest.mark.parametrize("n", [64, 128, 256, 512])
def test_fused_line_plan_with_pass_tables_is_the_filter(n):
    rng = np.random.default_rng(n)
    lines = 3
    x = rng.standard_normal((lines, n)) + 1j * rng.standard_normal((lines, n))
    f = rng.random(n) / n
    buf = np.zeros((lines, padi(n - 1) + 1), complex)  # padded scratch line
    cur, cur_padded = x.copy(), False
    for (R, NS, S, mid), tab in zip(passes(p2_plan(n)), tw_tables(n)):
        nR = n // R
        src = (lambda i: cur[:, padi(i)]) if cur_padded else (lambda i: cur[:, i])
        dst = np.zeros_like(buf)
        last = (not mid) and S > 0 and NS * R == n
        out = np.zeros((lines, n), complex) if last else dst
        for j in range(nR):
            k = j if mid else j % NS
            v = np.stack([src(j + r * nR) for r in range(R)], axis=-1)
            span = nR if mid else NS
            for r in range(1, R):
                if tab is not None:
                    v[:, r] *= tab[(r - 1) * span + k]
            if mid:
                v = dft(v, -1) * f[j + np.arange(R) * nR]
                v = dft(v, +1)
                idx = [j * R + q for q in range(R)]
            else:
                v = dft(v, S)
                o = (j // NS) * NS * R + k
                idx = [o + q * NS for q in range(R)]
            for q, i in enumerate(idx):
                if last:
                    out[:, i] = v[:, q]
                else:
                    out[:, padi(i)] = v[:, q]
        cur, cur_padded = out, not last
    want = np.fft.ifft(np.fft.fft(x, axis=1) * f, axis=1) * n
    assert np.max(np.abs(cur - want)) < 1e-12 * np.max(np.abs(want))


def plane_threads(n):
    # clv_launch.h plane_threads of the in-place form (FP32 planes of 64 take one thread
    # per line instead: test_radix_64_in_registers)
    return {32: 128, 96: 384, 128: 512}.get(n, n * n // 16)


def plane_plan(n):
    """clv_launch.h plane_fac: two radices, 12 a Good-Thomas 4 x 3 butterfly."""
    return {32: [8, 4], 64: [8, 8], 96: [12, 8], 128: [16, 8]}[n]


def plan_span(n, plan, p):
    """inplace_fft.cuh InPlace::span: L_p = n / (R_0 ... R_{p-1})."""
    L = n
    for r in plan[:p]:
        L //= r
    return L


def mid_freq(n, plan, j):
    """inplace_fft.cuh InPlace::mid_freq: the digits of j (place values L_{p+1} / R_last)
    reversed."""
    RL, rem, w, f = plan[-1], j, 1, 0
    for p in range(len(plan) - 1):
        S = plan_span(n, plan, p + 1) // RL
        q = rem // S
        rem -= q * S
        f += q * w
        w *= plan[p]
    return f


def butterflies(nl, n, R, T):
    """(line, j) of every butterfly of a pass, thread by thread: b = tid + p T < nl n / R."""
    nb = nl * (n // R)
    per = -(-nb // T)
    return [((tid + p * T) % nl, (tid + p * T) // nl) for tid in range(T) for p in range(per)
            if tid + p * T < nb]


def inplace_filter(view, n, plan, T, tw, f):
    """inplace_fft.cuh InPlace<Plan, n, NL, T>::filter (with pass 0) on the lines
    view[l, :] (NL = view.shape[0]).  In place: every butterfly reads and writes the same
    elements, and within a pass no two butterflies share one (checked), so the order of
    the butterflies is free."""
    nl = view.shape[0]
    NF = len(plan)

    def run_pass(R, body):
        touched = np.zeros((nl, n), int)
        for l, j in butterflies(nl, n, R, T):
            idx = body(l, j)
            touched[l, idx] += 1
        assert np.all(touched == 1)  # disjoint butterflies covering every line

    for p in range(NF - 1):  # forward passes (decimation in frequency)
        R, L = plan[p], plan_span(n, plan, p)
        S = L // R

        def dif(l, j, R=R, L=L, S=S):
            a0, k = (j // S) * L + j % S, j % S
            idx = [a0 + m * S for m in range(R)]
            y = dft(view[l, idx], -1)
            if S > 1:
                y = y * tw[np.arange(R) * k * (n // L)]
            view[l, idx] = y
            return idx
        run_pass(R, dif)
    RL, nR = plan[-1], n // plan[-1]

    def mid(l, j):
        idx = [j * RL + m for m in range(RL)]
        y = dft(view[l, idx], -1) * f[mid_freq(n, plan, j) + np.arange(RL) * nR]
        view[l, idx] = dft(y, +1)
        return idx
    run_pass(RL, mid)
    for p in range(NF - 2, -1, -1):  # inverse passes (decimation in time)
        R, L = plan[p], plan_span(n, plan, p)
        S = L // R

        def dit(l, j, R=R, L=L, S=S):
            a0, k = (j // S) * L + j % S, j % S
            idx = [a0 + q * S for q in range(R)]
            y = view[l, idx]
            if S > 1:
                y = y * np.conj(tw[np.arange(R) * k * (n // L)])
            view[l, idx] = dft(y, +1)
            return idx
        run_pass(R, dit)


def plane_lines_filter(t, n, tw, f, rows):
    """k_plane.cu: the plane's lines filtered in place, rows=True along each row (line
    l = row), else along each column (line l = column)."""
    inplace_filter(t if rows else t.T, n, plane_plan(n), plane_threads(n), tw, f)


def axis_tile_lines(n, esz):
    # clv_launch.h axis_tile_lines (esz: bytes of a real)
    w = 64 if n == 32 else (32 if n == 64 else (16 if n in (96, 128) else 8))
    return w // (1 if esz == 4 else 2)


@pytest.mark.parametrize("esz", [4, 8])
@pytest.mark.parametrize("n", [32, 64, 96, 128, 256, 512])
def test_in_place_axis_tile_is_the_filter(n, esz):
    """k_axis.cu in-place path: a full tile of W lines of a strided axis, 256 threads,
    the axis plans (8, 4, 2, 3, 5 in order; 128 = 16 x 8)."""
    W = axis_tile_lines(n, esz)
    rng = np.random.default_rng(n + esz)
    x = rng.standard_normal((W, n)) + 1j * rng.standard_normal((W, n))
    f = rng.random(n) / n
    tw = np.exp(-2j * np.pi * np.arange(n) / n)
    t = x.copy()
    inplace_filter(t, n, ax_plan(n), 256, tw, f)
    want = np.fft.ifft(np.fft.fft(x, axis=1) * f, axis=1) * n
    assert np.max(np.abs(t - want)) < 1e-12 * np.max(np.abs(want))


@pytest.mark.parametrize("S", [-1, 1])
def test_good_thomas_radix_12(S):
    """fft_radix.cuh Radix<12>: radix 4 over x[(3 n1 + 4 n2) mod 12], radix 3 across,
    outputs at (9 k1 + 4 k2) mod 12."""
    rng = np.random.default_rng(12)
    a = rng.standard_normal(12) + 1j * rng.standard_normal(12)
    y = np.array([dft(np.array([a[(3 * n1 + 4 * n2) % 12] for n1 in range(4)]), S) for n2 in range(3)])
    out = np.zeros(12, complex)
    for k1 in range(4):
        t = dft(y[:, k1], S)
        for k2 in range(3):
            out[(9 * k1 + 4 * k2) % 12] = t[k2]
    assert np.max(np.abs(out - dft(a, S))) < 1e-13


def cos64(m):
    """fft_radix.cuh cos64: a quarter-wave table and its symmetries."""
    quarter = [np.cos(2 * np.pi * k / 64) for k in range(16)] + [0.0]
    m &= 63
    if m <= 16:
        return quarter[m]
    if m <= 32:
        return -quarter[32 - m]
    if m <= 48:
        return -quarter[m - 32]
    return quarter[64 - m]


@pytest.mark.parametrize("S", [-1, 1])
def test_radix_64_in_registers(S):
    """fft_radix.cuh Radix<64>: radix 8 over x[8 n1 + n2], twiddle W64^(n2 k1) from
    cos64 / sin64 (sin64(m) = cos64(m - 16)), radix 8 across, outputs at k1 + 8 k2."""
    m = np.arange(64)
    assert np.allclose([cos64(k) for k in m], np.cos(2 * np.pi * m / 64), atol=1e-15)
    assert np.allclose([cos64((k + 48) & 63) for k in m], np.sin(2 * np.pi * m / 64), atol=1e-15)
    rng = np.random.default_rng(64)
    a = rng.standard_normal(64) + 1j * rng.standard_normal(64)
    y = np.zeros((8, 8), complex)
    for n2 in range(8):
        t = dft(np.array([a[8 * n1 + n2] for n1 in range(8)]), S)
        for k1 in range(8):
            q = n2 * k1
            y[n2, k1] = t[k1] * (cos64(q) + 1j * S * cos64((q + 48) & 63))
    out = np.zeros(64, complex)
    for k1 in range(8):
        t = dft(y[:, k1], S)
        for k2 in range(8):
            out[k1 + 8 * k2] = t[k2]
    assert np.max(np.abs(out - dft(a, S))) < 1e-12


def test_plane_lines_in_registers_64():
    """k_plane.cu plane_lines_in_registers: thread l loads column l (global a n + l), filters
    it with fr, stores it at tile[l + a PL]; then loads row l (tile[l PL + a]), filters it
    with fc cst, stores it back; the plane leaves in row order (dst[i n + l] = tile[i PL + l])."""
    n, PL = 64, 65
    rng = np.random.default_rng(65)
    g = rng.standard_normal(n * n) + 1j * rng.standard_normal(n * n)  # row-major plane
    fr, fc, cst = rng.random(n) / n, rng.random(n) / n, 0.8
    tile = np.zeros(n * PL, complex)
    for ph in (0, 1):
        f = fr if ph == 0 else fc * cst
        for l in range(n):
            v = g[np.arange(n) * n + l] if ph == 0 else tile[l * PL + np.arange(n)]
            v = dft(dft(v, -1) * f, +1)
            s0, sa = (l * PL, 1) if ph else (l, PL)
            tile[s0 + np.arange(n) * sa] = v
    dst = np.array([tile[i * PL + l] for i in range(n) for l in range(n)])
    x = g.reshape(n, n)
    want = np.fft.ifft(np.fft.fft(x, axis=0) * fr[:, None], axis=0) * n
    want = np.fft.ifft(np.fft.fft(want, axis=1) * (fc * cst), axis=1) * n
    assert np.max(np.abs(dst - want.reshape(-1))) < 1e-12 * np.max(np.abs(want))


def test_axis_line_addresses_partition_the_slice():
    """k_axis.cu axis_line_kernel: lane w of a tile (l0, nl) of a strided axis reads
    off + a inner (off = (l0 / inner) n inner + l0 mod inner + w); the engine's tiles
    (nl = min(W, inner - l0 mod inner)) cover every element of the slice exactly once."""
    for n, inner, lines in ((64, 4096, 4096), (64, 32, 32), (64, 48, 96)):
        W = 32
        seen = np.zeros(n * lines, int)
        l0 = 0
        while l0 < lines:
            nl = min(W, inner - l0 % inner)
            for w in range(nl):
                off = (l0 // inner) * n * inner + l0 % inner + w
                seen[off + np.arange(n) * inner] += 1
            l0 += nl
        assert np.all(seen == 1)


@pytest.mark.parametrize("n", [32, 64, 96, 128])
def test_in_place_plane_passes_are_the_2d_filter(n):
    rng = np.random.default_rng(n + 1)
    x = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    fr, fc = rng.random(n) / n, rng.random(n) / n
    tw = np.exp(-2j * np.pi * np.arange(n) / n)
    t = x.copy()
    plane_lines_filter(t, n, tw, fr, rows=False)  # along the columns (the slower axis) first
    plane_lines_filter(t, n, tw, fc, rows=True)
    want = np.fft.ifft(np.fft.fft(x, axis=1) * fc, axis=1) * n
    want = np.fft.ifft(np.fft.fft(want, axis=0) * fr[:, None], axis=0) * n
    assert np.max(np.abs(t - want)) < 1e-12 * np.max(np.abs(want))

"""Learned coarse solver: the MLP kernels against the CPU oracle (oracle/mlp_oracle.py),
the FP32 plain step against the FP64 step, the guard, and a training run that must beat
the plain coarse step it corrects."""
import numpy as np
import pytest


def test_bf16_rounding_matches_torch():
    import torch
    from oracle import mlp_oracle as M
    x = np.random.default_rng(0).standard_normal(10000).astype(np.float32) * 10
    x[:4] = [0.0, -0.0, 1e-40, 3.0e38]
    want = torch.from_numpy(x).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    np.testing.assert_array_equal(M.bf16_bits(x), want)


def test_box_filter_conserves_totals():
    from hyperflow_gb300.learned import box_filter
    U = np.random.default_rng(1).uniform(0.1, 2.0, (4, 64, 64))
    F = box_filter(U, 4)
    assert F.shape == (4, 16, 16)
    np.testing.assert_allclose(F.sum(axis=(1, 2)) * 16, U.sum(axis=(1, 2)), rtol=1e-13)


def test_mlp_oracle_gradient_is_the_derivative():
    """Central differences confirm the oracle's backward formulas on the unrounded network
    (BF16 rounding of activations is piecewise constant, so the kernels' backward -- like
    any BF16 training -- passes it straight through)."""
    from oracle import mlp_oracle as M
    from hyperflow_gb300.learned import init_params
    rng = np.random.default_rng(2)
    p = init_params(3, out_scale=1.0).astype(np.float64)
    x = M.bf16_bits(rng.standard_normal((8, 64)).astype(np.float32))
    dy = rng.standard_normal((8, 4))
    g = M.backward(p, x, dy, rounding=False)
    for k in (M.OFF_B3 + 1, M.OFF_W3 + 70, M.OFF_B2 + 5, M.OFF_W2 + 300, M.OFF_B1 + 7, M.OFF_W1 + 1234):
        e = np.zeros_like(p)
        e[k] = 1e-5
        fp = (M.forward(p + e, x, rounding=False)[0] * dy).sum()
        fm = (M.forward(p - e, x, rounding=False)[0] * dy).sum()
        assert abs((fp - fm) / 2e-5 - g[k]) < 1e-6 * (1 + abs(g[k]))


def _rand_case(rng, nf=1000):
    from oracle import mlp_oracle as M
    from hyperflow_gb300.learned import init_params
    p = init_params(int(rng.integers(100)), out_scale=1.0)
    p[M.OFF_B1:M.OFF_W2] = rng.uniform(-0.5, 0.5, 64)
    p[M.OFF_B3:] = rng.uniform(-0.1, 0.1, 4)
    x = M.bf16_bits(rng.standard_normal((nf, 64)).astype(np.float32))
    return p, x


@pytest.mark.gpu
def test_mlp_forward_on_tensor_cores_matches_oracle():
    from oracle import mlp_oracle as M
    from hyperflow_gb300.learned import LearnedSolver
    rng = np.random.default_rng(4)
    ls = LearnedSolver(300, 1 / 300)   # room for 180,600 faces
    # partial tiles, a full grid's faces, and more 256-face tiles than the kernel has CTAs (at
    # most 4 per SM), so that CTAs walk several tiles, the last one partial
    for nf in (1000, 17, 2 * 65 * 64, 160_000 + 77):
        p, x = _rand_case(rng, nf)
        ls.set_params(p)
        y = ls.mlp_forward(x)
        ref, _ = M.forward(p, x)
        # FP32 accumulation order, and GELU's tanh taken from the hardware approximation
        # (absolute error about 2^-11) where the oracle has numpy's: now and then a hidden
        # activation rounds to the neighbouring BF16 value, which moves the outputs by up to a
        # few 1e-3.  So: BF16-level agreement for all but a few in 10^4 outputs, every output
        # within 2e-2, and a small mean (a wrong tile or face would break all three)
        d = np.abs(y - ref)
        assert np.isfinite(y).all()
        assert (d <= 4e-3 + 2e-2 * np.abs(ref)).mean() >= 0.9999, d.max()
        assert d.max() < 2e-2 and d.mean() < 1e-3, (d.max(), d.mean())


@pytest.mark.gpu
@pytest.mark.parametrize("n", [37, 48])
def test_features_match_oracle_bit_for_bit(n):
    """The network's inputs (4x4 primitive stencil per face, scaled, BF16) and the correction
    scale: the GPU kernels against the oracle's float32 restatement, bit for bit, on a state
    after a few plain steps of a four-quadrant problem (n = 37: a partial last CTA of faces)."""
    from oracle import mlp_oracle as M
    from hyperflow_gb300 import CartSolver, cases
    from hyperflow_gb300.learned import LearnedSolver
    c = cases.quadrant_case(n, scheme="MUSCLHancock", limiter="MinBee", cfl=cases.CFL_2D)
    U = CartSolver(c).state(0)[:, 2:-2, 2:-2].astype(np.float32)
    ls = LearnedSolver(n, 1.0 / n, cfl=cases.CFL_2D)
    ls.set_state(U)
    for _ in range(6):
        ls.step(ls.cfl_dt(), False)
    x, sc = ls.features()
    xr, scr = M.features(ls.state(), 1.4)
    np.testing.assert_array_equal(sc, scr)
    np.testing.assert_array_equal(x, xr)


@pytest.mark.gpu
def test_mlp_backward_matches_oracle():
    from oracle import mlp_oracle as M
    from hyperflow_gb300.learned import LearnedSolver
    rng = np.random.default_rng(5)
    ls = LearnedSolver(64, 1 / 64)
    p, x = _rand_case(rng, 777)
    ls.set_params(p)
    dy = rng.standard_normal((777, 4)).astype(np.float32)
    g = ls.mlp_backward(x, dy)
    ref = M.backward(p, x, dy)
    for a, b in ((M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2), (M.OFF_B2, M.OFF_W3),
                 (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.NPARAM)):
        err = np.linalg.norm(g[a:b] - ref[a:b]) / (np.linalg.norm(ref[a:b]) + 1e-12)
        assert err < 2e-2, (a, b, err)


@pytest.mark.gpu
def test_fp32_plain_step_tracks_fp64_step():
    """The learned solver's plain FP32 path is the reference scheme in single precision."""
    from hyperflow_gb300 import CartSolver, cases
    from hyperflow_gb300.learned import LearnedSolver
    case = cases.quadrant_case(96, scheme="MUSCLHancock", limiter="MinBee")
    s = CartSolver(case)
    U0 = s.state(0)[:, 2:-2, 2:-2]
    ls = LearnedSolver(96, 1 / 96)
    ls.set_state(U0.astype(np.float32))
    for _ in range(20):
        dt = s.step()
        ls.step(dt, use_mlp=False)
    U = s.state(0)[:, 2:-2, 2:-2]
    V = ls.state().astype(np.float64)
    assert np.abs(V - U).max() / np.abs(U).max() < 2e-4


@pytest.mark.gpu
def test_guard_keeps_positivity_and_rejects():
    from oracle import mlp_oracle as M
    from hyperflow_gb300 import CartSolver, cases
    from hyperflow_gb300.learned import LearnedSolver, init_params
    case = cases.shock_bubble_case(128)
    s = CartSolver(case)
    U0 = s.state(0)[:, 2:-2, 2:-2].astype(np.float32)
    ls = LearnedSolver(128, 1 / 128)
    p = init_params(0)
    p[M.OFF_B3:] = [5.0, -5.0, 5.0, -50.0]          # absurd corrections
    ls.set_params(p)
    ls.set_state(U0)
    rejected = 0
    for _ in range(10):
        rejected += ls.step(ls.cfl_dt(), use_mlp=True)
    U = ls.state().astype(np.float64)
    rho = U[0]
    pres = 0.4 * (U[3] - 0.5 * (U[1] ** 2 + U[2] ** 2) / rho)
    assert rejected > 0 and (rho > 0).all() and (pres > 0).all()


@pytest.mark.gpu
@pytest.mark.parametrize("n,mode,ctas", [(37, 0, 0), (128, 0, 2), (128, 1, 1), (300, 0, 0), (300, 1, 3)])
def test_fused_face_kernel_equals_the_separate_kernels(n, mode, ctas):
    """An inference step with the features, MLP and corrections in one kernel per 256-face tile
    (and with the plain flux in it too) against the separate kernels (plain flux, features, MLP
    forward, correction): states and rejection counts equal bit for bit over steps of a
    shock-bubble flow with corrections large enough that the guard rejects some, in both guard
    modes (n = 37: a partial last tile; n = 300 at 1 CTA per SM: more tiles than CTAs)."""
    from oracle import mlp_oracle as M
    from hyperflow_gb300 import CartSolver, cases
    from hyperflow_gb300.learned import LearnedSolver, init_params
    s = CartSolver(cases.shock_bubble_case(n))
    s.run(10)
    U0 = s.state(0)[:, 2:-2, 2:-2].astype(np.float32)
    s.close()
    p = init_params(3, out_scale=0.05)
    p[M.OFF_B3:] = [0.05, -0.03, 0.04, -0.2]
    runs = []
    for fused in (0, 1, 2):
        ls = LearnedSolver(n, 1.0 / n)
        ls.set_params(p)
        ls.set_guard_mode(mode)
        ls.set_fused(fused, ctas)
        ls.set_state(U0)
        rej = [ls.step(ls.cfl_dt(), use_mlp=True) for _ in range(8)]
        runs.append((ls.state(), rej))
        ls.close()
    Ua, ra = runs[0]
    assert sum(ra) > 0 and sum(ra) < 8 * n * n, ra
    for Ub, rb in runs[1:]:
        assert ra == rb
        np.testing.assert_array_equal(Ua.view(np.uint32), Ub.view(np.uint32))


@pytest.mark.gpu
def test_local_extremum_guard_keeps_the_bounds():
    """Guard mode 1: after a step with absurd corrections, every cell's density and energy lie
    within the min / max over its 3x3 neighbourhood of the old state and the plain update."""
    from oracle import mlp_oracle as M
    from hyperflow_gb300 import CartSolver, cases
    from hyperflow_gb300.learned import LearnedSolver, init_params
    s = CartSolver(cases.shock_bubble_case(128))
    s.run(30)
    U0 = s.state(0)[:, 2:-2, 2:-2].astype(np.float32)
    ls = LearnedSolver(128, 1 / 128)
    p = init_params(0)
    p[M.OFF_B3:] = [0.5, -0.3, 0.4, -2.0]
    ls.set_params(p)
    ls.set_guard_mode(1)
    ls.set_state(U0)
    dt = ls.cfl_dt()
    ls.step(dt, use_mlp=False)
    Up = ls.state()
    ls.set_state(U0)
    rejected = ls.step(dt, use_mlp=True)
    U1 = ls.state()
    assert rejected > 0
    assert not np.array_equal(U1, Up)              # some corrections were kept
    for v in (0, 3):
        both = np.stack([U0[v], Up[v]])
        pad_lo = np.pad(both.min(0), 1, mode="edge")
        pad_hi = np.pad(both.max(0), 1, mode="edge")
        lo = np.min([pad_lo[1 + a:129 + a, 1 + b:129 + b] for a in (-1, 0, 1) for b in (-1, 0, 1)], axis=0)
        hi = np.max([pad_hi[1 + a:129 + a, 1 + b:129 + b] for a in (-1, 0, 1) for b in (-1, 0, 1)], axis=0)
        assert (U1[v] >= lo).all() and (U1[v] <= hi).all()


@pytest.mark.gpu
def test_training_beats_the_plain_coarse_step():
    """Trained on filtered 256^2 FP64 runs (4x coarser grid: 64^2), the corrected one-step
    error on held-out pairs is below the plain coarse step's -- what the network gains."""
    from hyperflow_gb300 import cases
    from hyperflow_gb300.learned import LearnedSolver, fine_pairs, init_params, one_step_loss, train
    tr = fine_pairs(cases.shock_bubble_case(256, t_end=1.0), 0.12, stride=2)
    tr += fine_pairs(cases.quadrant_case(256, scheme="MUSCLHancock", limiter="MinBee"), 0.06, stride=2)
    held = fine_pairs(cases.shock_bubble_case(256, bubble=(0.45, 0.55), radius=0.18, t_end=1.0), 0.1, stride=3)
    ls = LearnedSolver(64, 1 / 64)
    ls.set_params(init_params(0))
    losses, w = train(ls, tr, iters=600, lr=2e-3)
    plain = one_step_loss(ls, held, w, use_mlp=False)
    learned = one_step_loss(ls, held, w, use_mlp=True)
    assert np.isfinite(losses).all()
    assert losses[-50:].mean() < losses[:50].mean()
    assert learned < 0.9 * plain, (learned, plain)


@pytest.mark.gpu
def test_coarsen_on_device_equals_box_filter():
    """hf_coarsen (the training-data filter formed on the device) against the host box filter."""
    from hyperflow_gb300 import CartSolver, cases
    from hyperflow_gb300.learned import box_filter
    s = CartSolver(cases.shock_bubble_case(128))
    s.run(20)
    g = s.block_dims(0)["ghost"]
    want = box_filter(s.state(0)[:, g:-g, g:-g], 4)
    got = s.coarsen(0, 4)
    assert got.dtype == np.float32 and got.shape == (4, 32, 32)
    np.testing.assert_allclose(got, want, rtol=2e-7, atol=1e-12)


@pytest.mark.gpu
def test_learned_solver_lowers_the_end_time_error_in_both_families():
    """What the trained network gains where it counts: the error at the end of a run.  Trained on
    4x box-filtered 256^2 FP64 runs of the plain solver (8 seeded four-quadrant Riemann problems, 8
    shock-bubble flows), the learned 64^2 solver (change guard, bound 2) ends with a lower L1
    density error against the filtered 256^2 solution than the plain coarse solver on held-out
    cases of both families: two Riemann seeds and two bubble placements it was not trained on.
    (Seen across training seeds: learned / plain error 0.65-0.90 on these four cases.)"""
    from hyperflow_gb300 import cases
    from hyperflow_gb300.learned import (LearnedSolver, change_weights, evaluate_learned, evaluate_plain,
                                         fine_sequence, init_params, train)
    nf, f = 256, 4

    def rp(seed):
        return lambda n: cases.random_quadrant_case(n, seed)

    def sb(b, r, t_end=1.0):
        return lambda n: cases.shock_bubble_case(n, bubble=b, radius=r, t_end=t_end)

    rng = np.random.default_rng(1)
    train_sets = [(rp(100 + k), None) for k in range(8)]
    for _ in range(8):
        b = (float(rng.uniform(0.35, 0.5)), float(rng.uniform(0.4, 0.6)))
        train_sets.append((sb(b, float(rng.uniform(0.15, 0.22))), 0.25))
    pairs = []
    for fn, t_end in train_sets:
        c = fn(nf)
        st, dts = fine_sequence(c, t_end if t_end is not None else c["simulation"]["t_end"], factor=f)
        pairs += [(st[k], st[k + 1], dts[k]) for k in range(len(dts))]
    ls = LearnedSolver(nf // f, f / nf)
    ls.set_params(init_params(0))
    losses, _ = train(ls, pairs, 6000, lr=2e-3, seed=0, w=change_weights(pairs))
    params = ls.params()
    ls.close()
    assert np.isfinite(losses).all()
    held = {"riemann_200": (rp(200), rp(200)(nf)["simulation"]["t_end"]),
            "riemann_201": (rp(201), rp(201)(nf)["simulation"]["t_end"]),
            "bubble_a": (sb((0.42, 0.55), 0.2, 0.2), 0.2), "bubble_b": (sb((0.38, 0.45), 0.17, 0.2), 0.2)}
    ratios = {}
    for name, (fn, t_end) in held.items():
        res, ref, U0 = evaluate_plain(fn, nf, t_end, factor=f)
        learned = evaluate_learned(t_end, params, ref, U0, bound=2.0)
        ratios[name] = learned["l1_rho"] / res["fp32_plain"]["l1_rho"]
    assert all(r < 0.97 for r in ratios.values()), ratios
    assert np.mean(list(ratios.values())) < 0.9, ratios


def test_feature_oracle_equals_a_per_face_restatement():
    """The oracle's vectorised features (what the GPU features are pinned to, bit for bit) against
    a face-by-face float32 restatement of the same definition on a small random state: the 4x4
    stencil with mirrored cells past the edges, x faces first, scaled by the reciprocals of the
    face's reference density, sound speed and pressure, rounded to BF16."""
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(11)
    n, g = 5, np.float32(1.4)
    U = np.empty((4, n, n), np.float32)
    U[0] = rng.uniform(0.5, 2.0, (n, n))
    U[1] = U[0] * rng.uniform(-0.5, 0.5, (n, n))
    U[2] = U[0] * rng.uniform(-0.5, 0.5, (n, n))
    U[3] = rng.uniform(2.0, 4.0, (n, n))
    x, sc = M.features(U, 1.4)

    def prim(j, i):
        def m(k):
            k = -1 - k if k < 0 else (2 * n - 1 - k if k >= n else k)
            return min(max(k, 0), n - 1)
        c = U[:, m(j), m(i)]
        r = c[0]
        u, v = c[1] / r, c[2] / r
        p = np.float32(1.4 - 1.0) * (c[3] - np.float32(0.5) * r * (u * u + v * v))   # gamma - 1 in double, as the kernels
        return r, u, v, p

    one = np.float32(1.0)
    faces = [(0, i, j) for j in range(n) for i in range(n + 1)] + [(1, i, j) for j in range(n + 1) for i in range(n)]
    assert len(faces) == x.shape[0] == 2 * n * (n + 1)
    for f, (d, i, j) in enumerate(faces):
        il, jl = (i - 1, j) if d == 0 else (i, j - 1)
        ni, nj, ti, tj = (1, 0, 0, 1) if d == 0 else (0, 1, 1, 0)
        rl, _, _, pl = prim(jl, il)
        rh, _, _, ph = prim(jl + nj, il + ni)
        rr, pr = np.float32(0.5) * (rl + rh), np.float32(0.5) * (pl + ph)
        cref = np.sqrt(np.maximum(g * pr / rr, np.float32(1e-12)))
        assert sc[f, 0] == rr and sc[f, 1] == cref
        row = []
        for a in (-1, 0, 1, 2):
            for b in (-1, 0, 1, 2):
                r, u, v, p = prim(jl + a * nj + b * tj, il + a * ni + b * ti)
                un, ut = (u, v) if d == 0 else (v, u)
                row += [r * (one / rr) - one, un * (one / cref), ut * (one / cref), p * (one / pr) - one]
        np.testing.assert_array_equal(x[f], M.bf16_bits(np.array(row, np.float32)))


@pytest.mark.gpu
@pytest.mark.parametrize("use_mlp", [False, True])
def test_run_to_equals_a_loop_with_fresh_cfl_passes(use_mlp):
    """hf_lc_run_to waits once per step and takes each dt from the wave-speed maximum the previous
    step's update left; a loop that re-uploads the state before every step makes each dt come
    from a fresh CFL pass instead.  Same step count, rejection count and state, bit for bit."""
    from oracle import mlp_oracle as M
    from hyperflow_gb300 import CartSolver, cases
    from hyperflow_gb300.learned import LearnedSolver, init_params
    n, t_end = 64, 0.02
    s = CartSolver(cases.shock_bubble_case(n))
    s.run(5)
    U0 = s.state(0)[:, 2:-2, 2:-2].astype(np.float32)
    s.close()
    p = init_params(3, out_scale=0.05)
    p[M.OFF_B3:] = [0.05, -0.03, 0.04, -0.2]
    a = LearnedSolver(n, 1.0 / n)
    a.set_params(p)
    a.set_state(U0)
    ka, ra = a.run_to(t_end, use_mlp)
    b = LearnedSolver(n, 1.0 / n)
    b.set_params(p)
    b.set_state(U0)
    kb = rb = 0
    t = 0.0
    while t < t_end:
        b.set_state(b.state(), t)          # forgets the cached maximum
        dt = b.cfl_dt()
        if kb < 5:
            dt *= 0.2
        if t + dt > t_end:
            dt = t_end - t
        rb += b.step(dt, use_mlp)
        t += dt
        kb += 1
    assert ka == kb and ka > 10 and ra == rb and (ra > 0) == use_mlp
    np.testing.assert_array_equal(a.state().view(np.uint32), b.state().view(np.uint32))
    a.close()
    b.close()

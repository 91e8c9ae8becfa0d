"""The adjoint: gradients of the best-path log-likelihood along the fixed path.

CPU (no GPU): the FP64 oracle gradient against central finite differences
(h = 1e-3) of the same fixed path's score, and the path score rebuilt from the
path against the forward's best score (which pins the rule for which cells
carry an emission).  GPU: the adjoint kernel through the C ABI against the FP64
oracle gradient, a torch.autograd.Function over the ABI (checks only), and the
Gauss-Newton recalibration of perturbed scalings."""
import dataclasses
import math

import numpy as np
import pytest

from conftest import abea

H = 1e-3        # central-difference step
FD_RTOL = 1e-3  # finite differences vs the analytic FP64 gradient


def read_of(batch, i):
    seq = bytes(batch.read[batch.read_ptr[i]:batch.read_ptr[i] + batch.read_len[i]])
    ev = batch.events[batch.event_ptr[i]:batch.event_ptr[i] + batch.n_events[i]]
    return seq, ev


def penalties(n_events, n_kmers):
    """f5c's transition log-probabilities (GPU/align_cuda.cl:624-640)."""
    epk = n_events / n_kmers
    p_stay = 1 - 1 / (epk + 1)
    lp_skip = math.log(1e-10)
    lp_stay = math.log(p_stay)
    lp_step = math.log(1.0 - math.exp(lp_skip) - math.exp(lp_stay))
    return lp_step, lp_stay, lp_skip, math.log(0.01)


def moves(walk, last_from):
    """Move into each walked cell: 0 = D, 1 = U, 2 = L."""
    out = []
    for j in range(len(walk)):
        if j + 1 < len(walk):
            de = walk[j]["read_pos"] - walk[j + 1]["read_pos"]
            dk = walk[j]["ref_pos"] - walk[j + 1]["ref_pos"]
            out.append(0 if (de, dk) == (1, 1) else 1 if (de, dk) == (1, 0) else 2)
        else:
            out.append(last_from)
    return out


@pytest.fixture(scope="module")
def small_reads():
    from abea_gb300 import synth
    return synth.make_batch("adjoint", seed=11, lengths=[400, 650, 900, 1200])


def test_path_score_rebuilds_the_best_score(oracle_mod, small_reads):
    b = small_reads
    for i in range(b.n_reads):
        seq, ev = read_of(b, i)
        for flags in (0, oracle_mod.VAR_AWARE):
            _, _, info = oracle_mod.align(seq, ev, b.model, b.scalings[i], flags)
            walk, lf = info["walk"], info["last_from"]
            assert len(walk) == info["path_len"] > 0
            em, _, _, _ = oracle_mod.path_adjoint(walk, lf, seq, ev, b.model, b.scalings[i], flags)
            step, stay, skip, trim = penalties(len(ev), len(seq) - 5)
            s = em + sum((step, stay, skip)[m] for m in moves(walk, lf))
            e0, k0 = int(walk[-1]["read_pos"]), int(walk[-1]["ref_pos"])
            pe, pk = {0: (e0 - 1, k0 - 1), 1: (e0 - 1, k0), 2: (e0, k0 - 1)}[lf]
            assert pk == -1  # the walk ends on the trim column
            s += trim * (pe + 1)
            s += (len(ev) - info["best_event"]) * trim
            # the forward sums in FP32 cell by cell; a misplaced emission or
            # transition would be off by >= 0.5
            assert abs(s - info["best_score"]) <= 1e-4 * abs(s), (i, flags, s, info["best_score"])


@pytest.mark.parametrize("flags", [0, 4])
def test_oracle_gradient_matches_central_differences(oracle_mod, small_reads, flags):
    b = small_reads
    for i in range(b.n_reads):
        seq, ev = read_of(b, i)
        sc = b.scalings[i]
        _, _, info = oracle_mod.align(seq, ev, b.model, sc, flags)
        walk, lf = info["walk"], info["last_from"]
        _, g, _, gm = oracle_mod.path_adjoint(walk, lf, seq, ev, b.model, sc, flags, want_model=True)
        theta0 = np.array([sc["shift"], sc["scale"], sc["var"]], dtype=np.float64)

        def f(theta=None, **kw):
            return oracle_mod.path_adjoint(walk, lf, seq, ev, b.model, sc, flags, theta=theta, **kw)[0]

        for p in range(3):
            tp, tm = theta0.copy(), theta0.copy()
            tp[p] += H
            tm[p] -= H
            fd = (f(tp) - f(tm)) / (2 * H)
            if flags == 0 and p == 2:
                assert g[2] == 0.0 and fd == 0.0  # var is not used by the parity emission
                continue
            assert abs(fd - g[p]) <= FD_RTOL * max(abs(g[p]), 1.0), (i, p, fd, g[p])
        # a few k-mers on the path: level_mean and level_stdv
        used = np.nonzero(np.any(gm != 0, axis=1))[0]
        for k in used[:: max(1, len(used) // 6)]:
            for which in ("d_mean", "d_stdv"):
                fd = (f(kmer=int(k), **{which: H}) - f(kmer=int(k), **{which: -H})) / (2 * H)
                ga = gm[k, 0 if which == "d_mean" else 1]
                assert abs(fd - ga) <= FD_RTOL * max(abs(ga), 1.0), (i, k, which, fd, ga)


def test_oracle_gauss_newton_step_is_exact_on_a_fixed_path(oracle_mod, small_reads):
    """The residuals are linear in (shift, scale): after one GN step the fixed-path
    gradient in (shift, scale) vanishes."""
    b = small_reads
    seq, ev = read_of(b, 3)
    sc = b.scalings[3].copy()
    _, _, info = oracle_mod.align(seq, ev, b.model, sc)
    walk, lf = info["walk"], info["last_from"]
    _, g0, h, _ = oracle_mod.path_adjoint(walk, lf, seq, ev, b.model, sc)
    A = np.array([[h[0], h[1]], [h[1], h[2]]])
    d = np.linalg.solve(A, -np.array([h[3], h[4]]))
    theta = np.array([sc["shift"] + d[0], sc["scale"] + d[1], sc["var"]], dtype=np.float64)
    _, g1, _, _ = oracle_mod.path_adjoint(walk, lf, seq, ev, b.model, sc, theta=theta)
    assert np.all(np.abs(g1[:2]) <= 1e-8 * np.abs(g0[:2]).max() + 1e-9)


# ------------------------------------------------------------------------- GPU
def oracle_adjoint(oracle_mod, batch, flags):
    n = batch.n_reads
    g = np.zeros((n, 3))
    em = np.zeros(n)
    gm = np.zeros((4096, 2))
    lens = np.zeros(n, dtype=np.int64)
    for i in range(n):
        seq, ev = read_of(batch, i)
        if len(seq) < 6 or len(ev) == 0:
            continue
        _, _, info = oracle_mod.align(seq, ev, batch.model, batch.scalings[i], flags)
        walk, lf = info["walk"], info["last_from"]
        lens[i] = len(walk)
        em[i], g[i], _, gmi = oracle_mod.path_adjoint(walk, lf, seq, ev, batch.model, batch.scalings[i], flags,
                                                      want_model=True)
        gm += gmi
    return g, em, gm, lens


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [abea.MODE_PLAIN, abea.MODE_BATCHED])
@pytest.mark.parametrize("var_aware", [0, 1])
def test_gpu_adjoint_matches_fp64_oracle(oracle_mod, mode, var_aware):
    from abea_gb300 import synth
    batch = synth.make_batch("small", seed=21)
    flags = oracle_mod.VAR_AWARE if var_aware else 0
    ctx = abea.Context(0, mode)
    ctx.set_option(abea.OPT_VAR_AWARE, var_aware)
    dev = ctx.upload(batch)
    dev.run()
    gp, gc = dev.results()
    # the var-aware forward is bit-exact against the oracle's var-aware mode too
    op, oc, _ = oracle_mod.align_batch(batch, flags)
    assert np.array_equal(gc, oc)
    got = abea.split_pairs(batch, gp, gc)
    exp = abea.split_pairs(batch, op, oc)
    assert all(np.array_equal(x, y) for x, y in zip(got, exp))
    out = dev.backward()
    assert np.all(out["status"] == 0)
    g, em, gm, lens = oracle_adjoint(oracle_mod, batch, flags)
    # the same FP64 terms summed in another order: equal to the rounding of the sums
    tol = 1e-9 * (np.abs(g) + 100.0 * lens[:, None])
    assert np.all(np.abs(out["grad_scalings"] - g) <= tol), np.abs(out["grad_scalings"] - g).max()
    assert np.all(np.abs(out["path_emission"] - em) <= 1e-9 * (np.abs(em) + 100.0 * lens))
    assert np.allclose(out["grad_model"], gm, rtol=1e-9, atol=1e-9)
    assert np.count_nonzero(gm[:, 1]) > 1000
    if not var_aware:
        assert np.all(out["grad_scalings"][:, 2] == 0.0)


@pytest.mark.gpu
def test_gpu_adjoint_through_autograd(oracle_mod):
    """A torch.autograd.Function over the C ABI (for this check only): the
    gradient of sum(w * path_emission) w.r.t. (shift, scale, var) is w * the
    adjoint, and matches central differences of the oracle's fixed-path score."""
    import torch
    from abea_gb300 import synth

    batch = synth.make_batch("adjoint", seed=5, lengths=[1500, 2500, 4000, 700, 3300, 5000])
    ctx = abea.Context(0, abea.MODE_BATCHED)
    ctx.set_option(abea.OPT_VAR_AWARE, 1)
    dev = ctx.upload(batch)

    class PathScore(torch.autograd.Function):
        @staticmethod
        def forward(fctx, theta):
            sc = batch.scalings.copy()
            t = theta.detach().cpu().numpy()
            sc["shift"], sc["scale"], sc["var"] = t[:, 0], t[:, 1], t[:, 2]
            sc["log_var"] = np.log(t[:, 2]).astype(np.float32)
            dev.set_scalings(sc)
            dev.run()
            dev.sync()
            out = dev.backward(model_grad=False)
            fctx.save_for_backward(torch.from_numpy(out["grad_scalings"].copy()))
            return torch.from_numpy(out["path_emission"].copy())

        @staticmethod
        def backward(fctx, grad_out):
            (g,) = fctx.saved_tensors
            return grad_out[:, None] * g

    theta0 = np.stack([batch.scalings["shift"], batch.scalings["scale"], batch.scalings["var"]], 1)
    theta = torch.tensor(theta0.astype(np.float64), requires_grad=True)
    w = torch.linspace(0.5, 1.5, batch.n_reads, dtype=torch.float64)
    loss = (w * PathScore.apply(theta)).sum()
    loss.backward()
    for i in range(batch.n_reads):
        seq, ev = read_of(batch, i)
        _, _, info = oracle_mod.align(seq, ev, batch.model, batch.scalings[i], oracle_mod.VAR_AWARE)
        walk, lf = info["walk"], info["last_from"]
        t0 = np.array([batch.scalings[i]["shift"], batch.scalings[i]["scale"], batch.scalings[i]["var"]],
                      dtype=np.float64)
        for p in range(3):
            tp, tm = t0.copy(), t0.copy()
            tp[p] += H
            tm[p] -= H
            fp = oracle_mod.path_adjoint(walk, lf, seq, ev, batch.model, batch.scalings[i], oracle_mod.VAR_AWARE,
                                         theta=tp)[0]
            fm = oracle_mod.path_adjoint(walk, lf, seq, ev, batch.model, batch.scalings[i], oracle_mod.VAR_AWARE,
                                         theta=tm)[0]
            fd = float(w[i]) * (fp - fm) / (2 * H)
            ga = float(theta.grad[i, p])
            assert abs(fd - ga) <= FD_RTOL * max(abs(ga), 1.0), (i, p, fd, ga)


@pytest.mark.gpu
def test_gpu_recalibration_recovers_perturbed_scalings():
    """Scalings off by up to 8 pA and 10%: three annealed Gauss-Newton rounds
    bring shift within 1 pA and scale within 1% for nearly every read."""
    from abea_gb300 import synth
    rng = np.random.default_rng(4)
    batch = synth.make_batch("adjoint", seed=9, perturb=True, lengths=rng.integers(1000, 10001, 96))
    true = batch.meta["true_scalings"]
    ctx = abea.Context(0, abea.MODE_BATCHED)
    dev = ctx.upload(batch)
    before_shift = np.abs(batch.scalings["shift"] - true["shift"])
    sc = dev.recalibrate(3, first_temperature=5.0)
    ds = np.abs(sc["shift"] - true["shift"])
    dk = np.abs(sc["scale"] / true["scale"] - 1)
    ok = (ds < 1.0) & (dk < 0.01)
    assert np.median(before_shift) > 2.0
    assert ok.mean() >= 0.9, (ok.mean(), np.median(ds), np.median(dk))
    assert np.median(ds) < 0.5 and np.median(dk) < 0.005
    # the batch is left aligned with the final scalings: same as a fresh run with them
    gp, gc = dev.results()
    b2 = dataclasses.replace(batch, scalings=sc)
    ctx2 = abea.Context(0, abea.MODE_PLAIN)
    p2, c2 = ctx2.align_batch(b2)
    assert np.array_equal(gc, c2)
    for x, y in zip(abea.split_pairs(batch, gp, gc), abea.split_pairs(b2, p2, c2)):
        assert np.array_equal(x, y)

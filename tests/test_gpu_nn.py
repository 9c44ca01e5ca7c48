"""The learned initial guess on the GPU.

* Gradients of the library's network kernels (fp16 tensor-core GEMMs) against
  the float64 oracle of the same network (oracle/nn_oracle.py, itself pinned by
  finite differences).
* Training on solver-generated pairs lowers the loss, and on held-out scenes
  the network's prediction makes GMRES converge in fewer iterations than a zero
  start, to an answer within 1e-6 of the dense solve (the judge).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _random_batch(G, B, seed):
    rng = np.random.default_rng(seed)
    V = G ** 3
    mask = (rng.random((B, V)) < 0.5).astype(np.float32)
    inp = (rng.standard_normal((B, V, 16)) * 0.5).astype(np.float32)
    inp[:, :, :2] *= mask[:, :, None]
    tgt = (inp[:, :, 2:8] + 0.3 * rng.standard_normal((B, V, 6))).astype(np.float32)
    return inp, mask, tgt


def test_gradients_match_oracle(gpulib):
    from midas_gb300.learned import Net
    from midas_gb300.solver import Context
    from oracle import nn_oracle as N
    ctx = Context()
    G = 8
    net = Net(ctx, G, seed=3)
    theta = net.params().astype(np.float64)
    rng = np.random.default_rng(7)
    theta[:] = rng.standard_normal(len(theta)) * 0.08
    off = sum(co * 27 * ci + co for ci, co in zip(N.CI[:3], N.CO[:3]))
    theta[off + 6 * 27 * 32:off + 8 * 27 * 32] = 0      # padded output rows
    theta[off + 8 * 27 * 32 + 6:] = 0
    net.set_params(theta.astype(np.float32))
    inp, mask, tgt = _random_batch(G, 2, 1)
    loss = net.gradients(inp, mask, tgt)
    g = net.params(grads=True).astype(np.float64)
    loss_o, g_o = N.loss_and_grads(net.params().astype(np.float64), inp, mask, tgt, G, fp16=True)
    assert abs(loss - loss_o) <= 1e-4 * loss_o, (loss, loss_o)
    o = 0
    for (ws, bs) in N.param_shapes():
        n = int(np.prod(ws)) + bs[0]
        a, b = g[o:o + n], g_o[o:o + n]
        o += n
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
        print("layer", ws, "grad rel", rel, "cos", cos)
        assert rel < 5e-3 and cos > 0.99999
    net.close()
    ctx.close()


def test_gradients_match_oracle_at_training_size(gpulib):
    """The training configuration (16^3 grid, batch 8: 32,768 GEMM rows, more
    output tiles than the GPU has SMs) against the oracle."""
    from midas_gb300.learned import Net
    from midas_gb300.solver import Context
    from oracle import nn_oracle as N
    ctx = Context()
    G, B = 16, 8
    net = Net(ctx, G, seed=3)
    inp, mask, tgt = _random_batch(G, B, 11)
    loss = net.gradients(inp, mask, tgt)
    g = net.params(grads=True).astype(np.float64)
    loss_o, g_o = N.loss_and_grads(net.params().astype(np.float64), inp, mask, tgt, G, fp16=True)
    assert abs(loss - loss_o) <= 1e-4 * loss_o, (loss, loss_o)
    o = 0
    for (ws, bs) in N.param_shapes():
        n = int(np.prod(ws)) + bs[0]
        a, b = g[o:o + n], g_o[o:o + n]
        o += n
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
        print("layer", ws, "grad rel", rel, "cos", cos)
        assert rel < 1e-2 and cos > 0.9999   # fp16 operands summed over 32,768 voxels
    E = net.forward(inp, mask)
    params = N.unpack(net.params().astype(np.float64))
    X = N._f16(inp)
    for l, (W, b) in enumerate(params):
        z = N.conv(X, N._f16(W), G) + b
        X = N._f16(np.maximum(z, 0)) if l < 3 else z
    ref = inp[:, :, 2:8] + mask[:, :, None] * X[:, :, :6]
    assert np.max(np.abs(E - ref)) <= 1e-3 * max(1.0, np.max(np.abs(ref)))
    net.close()
    ctx.close()


def test_adam_steps_follow_the_oracle(gpulib):
    """Five training steps of the library (gradients, Adam, fp16 weight copies)
    against Adam on the oracle's gradients from the same start."""
    from midas_gb300.learned import Net
    from midas_gb300.solver import Context
    from oracle import nn_oracle as N
    ctx = Context()
    G = 8
    net = Net(ctx, G, seed=9)
    inp, mask, tgt = _random_batch(G, 2, 5)
    theta = net.params().astype(np.float64)
    live = np.ones_like(theta)
    off = sum(co * 27 * ci + co for ci, co in zip(N.CI[:3], N.CO[:3]))
    live[off + 6 * 27 * 32:off + 8 * 27 * 32] = 0
    live[off + 8 * 27 * 32 + 6:] = 0
    m = np.zeros_like(theta)
    v = np.zeros_like(theta)
    lr, b1, b2, eps = 1e-2, 0.9, 0.999, 1e-8
    losses = []
    for k in range(1, 6):
        loss = net.train_step(inp, mask, tgt, lr)
        loss_o, g = N.loss_and_grads(theta, inp, mask, tgt, G, fp16=True)
        assert abs(loss - loss_o) <= 2e-3 * loss_o, (k, loss, loss_o)
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        step = lr * (m / (1 - b1 ** k)) / (np.sqrt(v / (1 - b2 ** k)) + eps) * live
        got = net.params().astype(np.float64)
        cos = (theta - got) @ step / (np.linalg.norm(theta - got) * np.linalg.norm(step))
        print("step", k, "loss", loss, loss_o, "update cosine", cos)
        assert cos > 0.99
        assert np.all(got[live == 0] == 0)
        theta = got   # the next oracle step starts where the library is
        losses.append(loss)
    assert losses[-1] < losses[0]
    net.close()
    ctx.close()


def test_forward_prediction_is_incident_field_plus_masked_output(gpulib):
    from midas_gb300.learned import Net
    from midas_gb300.solver import Context
    from oracle import nn_oracle as N
    ctx = Context()
    net = Net(ctx, 8, seed=4)
    inp, mask, _ = _random_batch(8, 3, 2)
    E = net.forward(inp, mask)
    theta = net.params().astype(np.float64)
    params = N.unpack(theta)
    X = N._f16(inp)
    for l, (W, b) in enumerate(params):
        z = N.conv(X, N._f16(W), 8) + b
        X = N._f16(np.maximum(z, 0)) if l < 3 else z
    ref = inp[:, :, 2:8] + mask[:, :, None] * X[:, :, :6]
    assert np.max(np.abs(E - ref)) <= 1e-4 * max(1.0, np.max(np.abs(ref)))
    assert np.all(E[mask == 0] == inp[mask == 0][:, 2:8])
    net.close()
    ctx.close()


def test_guess_training_lowers_loss_and_saves_gmres_iterations(gpulib):
    """The initial-guess network trained on solver-generated pairs: the loss
    falls, and on held-out scenes GMRES from its prediction takes fewer
    iterations than from zero, to answers within 1e-6 of the dense solve."""
    from midas_gb300 import learned as LG
    from midas_gb300.solver import Context
    ctx = Context()
    G = 16
    data, its = LG.generate(ctx, LG.scenes(21, 64, G), tol=1e-6)
    assert len(data[0]) >= 100
    net = LG.Net(ctx, G, seed=5)
    hist = LG.train(net, data, epochs=30, batch=8, lr=1e-3)
    print("loss history", hist)
    assert hist[-1] < 0.5 * hist[0]
    rows = LG.evaluate(ctx, LG.scenes(99, 8, G), guess_net=net, tol=1e-8, judge=8)
    s = LG.summarise(rows)
    print(s)
    assert s["mean_its_guess"] < s["mean_its_zero"]
    assert s["converged_guess"] == s["scenes"] == s["converged_zero"]
    assert s["max_err_guess_vs_dense"] <= 1e-6 and s["max_err_zero_vs_dense"] <= 1e-6
    assert s["mean_err_guess_start_vs_dense"] < 1.0
    net.close()
    ctx.close()


def test_learned_preconditioner_cuts_fgmres_iterations(gpulib):
    """The preconditioner network trained on Krylov pairs (Z e, e) of 64 scenes:
    on held-out scenes flexible GMRES with it takes at most 85 % of the
    iterations of Jacobi-preconditioned GMRES, every answer accepted on its FP64
    true residual and within 1e-6 of the dense solve."""
    from midas_gb300 import learned as LG
    from midas_gb300.solver import Context
    ctx = Context()
    G = 16
    net = LG.Net(ctx, G, seed=6)
    pairs = LG.generate_prec(ctx, net, LG.scenes(31, 64, G), nvec=24)
    assert len(pairs) == 64 * 48
    hist = LG.train(net, pairs.as_data(), epochs=20, batch=16, lr=1e-3)
    print("loss history", hist)
    assert hist[-1] < 0.7 * hist[0]
    rows = LG.evaluate(ctx, LG.scenes(99, 8, G), prec_net=net, tol=1e-8, judge=8)
    s = LG.summarise(rows)
    print(s)
    assert s["converged_prec"] == s["scenes"] == s["converged_zero"]
    assert s["iteration_ratio_prec"] <= 0.85
    assert s["max_err_prec_vs_dense"] <= 1e-6 and s["max_err_zero_vs_dense"] <= 1e-6
    net.close()
    ctx.close()

"""GPU: the learned constitutive surrogate against its CPU oracle and against the exact step.

  - the training kernels' loss and gradients match oracle/mlp_oracle.py (FP32 and the BF16
    forward), and the tensor-core inference matches the oracle's BF16 forward;
  - captured tuples satisfy the Drucker-Prager flow rule (the oracle's scale-free target);
  - training on captured tuples lowers the loss;
  - with every prediction rejected the step is bit-identical to the FP32 form without the
    surrogate; with the trained network it stays within the FP32 form's error bar.
"""
import numpy as np
import pytest

import cases
import mlp_oracle as mo
import sps_gb300
from sps_gb300 import _abi
from sps_gb300 import surrogate as sg

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300)


def random_tuples(rng, n):
    x = rng.uniform(-1.0, 1.0, (n, mo.NIN))
    t = rng.uniform(-1.0, 1.0, (n, mo.NOUT))
    return np.concatenate([x, t], axis=1).astype(np.float32)


def layer_errors(g_gpu, g_ref):
    out = []
    for off, k, n in mo.LAYERS:
        sl = slice(off, off + k * n + n)
        out.append(rel_l2(g_gpu[sl], g_ref[sl]))
    return out


@pytest.mark.parametrize("quantize,tol", [(False, 1e-4), (True, 3e-3)])
def test_gradients_match_oracle(built_gpu, quantize, tol):
    rng = np.random.default_rng(3)
    net = sg.Mlp(batch=512, seed=7, quantize=quantize)
    p = net.params().astype(np.float64)
    t = random_tuples(rng, 500)
    loss, g = net.grad(t)
    loss_ref, g_ref = mo.loss_grad(p, t.astype(np.float64), quantize=quantize)
    assert abs(loss - loss_ref) <= tol * loss_ref, (loss, loss_ref)
    errs = layer_errors(g, g_ref)
    assert max(errs) <= tol, errs
    net.close()


@pytest.mark.parametrize("tensor_memory", [True, False], ids=["tcgen05", "mma_sync"])
def test_tensor_core_inference_matches_oracle(built_gpu, tensor_memory):
    # the tcgen05 path (128-row tiles, tensor-memory accumulators; 1000 rows: a ragged last
    # tile) and the warp-level mma.sync path against the oracle's BF16 forward pass
    rng = np.random.default_rng(4)
    net = sg.Mlp(batch=256, seed=11)
    net.set_inference(tensor_memory)
    p = net.params().astype(np.float64)
    x = rng.uniform(-1.0, 1.0, (1000, mo.NIN)).astype(np.float32)
    y = net.predict(x)
    y_ref, _ = mo.forward(p, x.astype(np.float64), quantize=True)
    assert rel_l2(y, y_ref) <= 5e-3, rel_l2(y, y_ref)
    # many tiles over every SM, and a second call on the same network
    x2 = rng.uniform(-1.0, 1.0, (200_000, mo.NIN)).astype(np.float32)
    y2_ref, _ = mo.forward(p, x2.astype(np.float64), quantize=True)
    for _ in range(2):
        y2 = net.predict(x2)
        assert rel_l2(y2, y2_ref) <= 5e-3, rel_l2(y2, y2_ref)
    net.close()


def _capture_column(precision, nsteps=40, cap=400000, **mat):
    prob = cases.column(dx=0.004, **mat)
    ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps", prob.params_copy(precision=precision))
    ctx.upload_problem(prob)
    sg.capture(ctx, cap)
    ctx.step(nsteps, 0.0)
    tuples, seen = sg.read_capture(ctx)
    ctx.close()
    return tuples, seen


def test_captured_tuples_follow_flow_rule(built_gpu):
    tuples, seen = _capture_column(_abi.SPS_PREC_FP64_PLAIN)
    assert len(tuples) > 1000 and seen == len(tuples)
    ref = mo.dp_target(tuples[:, :mo.NIN])
    # FP32 flow-rule body and FP32-rounded inputs
    assert rel_l2(tuples[:, mo.NIN:], ref) <= 1e-4, rel_l2(tuples[:, mo.NIN:], ref)
    # beyond the capacity tuples are dropped but still counted (the plain form is
    # deterministic, so the count is the same; the order of the tuples is not)
    tuples2, seen2 = _capture_column(_abi.SPS_PREC_FP64_PLAIN, cap=100)
    assert len(tuples2) == 100 and seen2 == seen
    held = {r.tobytes() for r in tuples}
    assert all(r.tobytes() in held for r in tuples2)


# material ranges of the training draws; the evaluation column sits inside them
RANGES = dict(phi_deg=(18, 34), cohesion=(0, 400), young=(4e6, 4e7), poiss=(0.22, 0.34),
              rho=(1900, 2700), k0=(0.3, 0.6))
EVAL_MATERIAL = dict(phi_deg=25.0, cohesion=150.0, young=1.5e7, poiss=0.28, rho=2300.0, k0=0.45)


def training_set(seed=0, ncol=6, nsteps=1500, every=15):
    """Tuples from column collapses with seeded, stratified material draws."""
    out = [sg.sample_run(cases.column(dx=0.004, **mat), _abi.SPS_PREC_FP32_FAST, nsteps, every)
           for mat in sg.stratified_materials(RANGES, ncol, seed)]
    return np.concatenate(out)


@pytest.fixture(scope="module")
def trained():
    data = training_set()
    rng = np.random.default_rng(9)
    idx = rng.permutation(len(data))
    hold = data[idx[:20000]]
    train = data[idx[20000:]]
    net = sg.Mlp(batch=4096, seed=5)
    net.set_data(train)
    loss = net.fit()
    return net, train, hold, loss


def test_training_lowers_loss(built_gpu, trained):
    net, train, hold, loss = trained
    assert len(train) >= 100000, len(train)
    assert loss[-1] < 0.2 * loss[0], loss
    y = net.predict(hold[:, :mo.NIN])
    err = rel_l2(y, hold[:, mo.NIN:].astype(np.float64))
    print("training tuples %d, loss per epoch %s, held-out relative L2 %.3g"
          % (len(train), np.array2string(loss, precision=3), err))
    assert err < 0.08


def _run(prob, nsteps, precision, net=None, tol=1e-6, env=None, gate=None, gate_steps=None):
    ctx = sps_gb300.StepContext(sps_gb300.gpu_lib(), "sps", prob.params_copy(precision=precision))
    ctx.upload_problem(prob)
    if net is not None:
        sg.install(ctx, net, tol=tol, envelope=env)
        if gate is not None:
            sg.set_gate(ctx, gate)
    ctx.step(nsteps, 0.0)
    out = ctx.download()
    st = sg.stats(ctx) if net is not None else None
    if gate_steps is not None:
        gate_steps.extend(sg.gate_stats(ctx))
    ctx.close()
    return out, st


def test_rejected_predictions_change_nothing(built_gpu, trained):
    net, train, _, _ = trained
    prob = cases.column(dx=0.004, **EVAL_MATERIAL)
    env = sg.Envelope.of(train)
    a, st = _run(prob, 40, _abi.SPS_PREC_FP32_FAST, net, tol=-1.0, env=env)
    b, _ = _run(prob, 40, _abi.SPS_PREC_FP32_FAST)
    for k in ("x", "vel", "stress", "f_drucker", "intvars1"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    loading, answered, outside, rejected = st
    assert loading > 0 and answered == 0 and outside + rejected == loading, st


def test_trained_surrogate_within_error_bar(built_gpu, trained):
    net, train, _, _ = trained
    prob = cases.column(dx=0.004, **EVAL_MATERIAL)
    env = sg.Envelope.of(train)
    nsteps = 200
    plain, _ = _run(prob, nsteps, _abi.SPS_PREC_FP64_PLAIN)
    fast, _ = _run(prob, nsteps, _abi.SPS_PREC_FP32_FAST)
    nt = prob.ntotal
    e_fast = rel_l2(fast["stress"][:4 * nt], plain["stress"][:4 * nt])
    for tol in (1e-6, 1e-4, 1e-2):
        # the gate off: the network runs in every step, so its effect on the error shows
        sur, st = _run(prob, nsteps, _abi.SPS_PREC_FP32_FAST, net, tol=tol, env=env, gate=0.0)
        e = rel_l2(sur["stress"][:4 * nt], plain["stress"][:4 * nt])
        ev = rel_l2(sur["vel"][:2 * nt], plain["vel"][:2 * nt])
        loading, answered, outside, rejected = st
        print("tol %.0e: loading %d, answered %.4f, outside envelope %.4f, drift-rejected "
              "%.4f; stress rel L2 vs FP64 %.3g (FP32 form alone %.3g), velocity %.3g"
              % (tol, loading, answered / loading, outside / loading, rejected / loading,
                 e, e_fast, ev))
        assert loading > 0
        if tol == 1e-6:
            assert e <= max(3.0 * e_fast, 1e-4), (e, e_fast)


def test_gate_skips_steps_where_the_network_does_not_answer(built_gpu, trained):
    # every prediction rejected (tol < 0): after the first step with loading evaluations the
    # gate closes, and it reopens for single steps at doubling intervals; the results stay
    # those of the FP32 form without the network
    net, train, _, _ = trained
    prob = cases.column(dx=0.004, **EVAL_MATERIAL)
    env = sg.Envelope.of(train)
    n = 60
    steps = []
    a, st = _run(prob, n, _abi.SPS_PREC_FP32_FAST, net, tol=-1.0, env=env, gate_steps=steps)
    b, _ = _run(prob, n, _abi.SPS_PREC_FP32_FAST)
    for k in ("x", "vel", "stress", "f_drucker", "intvars1"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    on, off = steps
    assert on + off == n and 3 <= on <= 8, steps
    assert st[0] > 0 and st[1] == 0
    # the gate off: the network runs in every step
    steps = []
    _run(prob, 20, _abi.SPS_PREC_FP32_FAST, net, tol=-1.0, env=env, gate=0.0, gate_steps=steps)
    assert steps == [20, 0]
    # steps that pass keep the network on (every prediction inside the envelope accepted,
    # a threshold that any answered evaluation meets); the first step has no loading
    # evaluation (no plasticity at time 0), so the gate is off in the second
    steps = []
    _, st = _run(prob, 20, _abi.SPS_PREC_FP32_FAST, net, tol=1e30, env=env, gate=1e-6,
                 gate_steps=steps)
    assert st[1] > 0 and steps == [19, 1], (st, steps)

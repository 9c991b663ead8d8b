"""Learned proposal of the energy-transfer draw (trekis_mlp_train, sampler = 1).

* Gradients of one training pass (tcgen05 products, BF16 operands, FP32
  accumulation) against a numpy restatement of the same network that rounds
  the same operands to BF16.
* Training lowers the loss, and the guess walks fewer brackets than the
  bisection probes.
* Exactness: the proposal only steers the bracket search, so a run with
  sampler = 1 gives the same draws, counts and tallies as sampler = 0, bit for
  bit, in FP64 and in FP32.
"""
import ctypes as C

import numpy as np
import pytest

from test_gpu_tc import bf16
from trekis import abi, api, configs

NP = 128 + 64 + 4096 + 64 + 64 + 1


def split(p):
    W1 = p[0:128].reshape(2, 64); b1 = p[128:192]; W2 = p[192:4288].reshape(64, 64)
    b2 = p[4288:4352]; w3 = p[4352:4416]; b3 = p[4416]
    return W1, b1, W2, b2, w3, b3


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def reference_grad(p, X, T):
    """Mean-squared-error gradient with the kernels' BF16 rounding of every
    tensor-core operand; elementwise work in float64."""
    W1, b1, W2, b2, w3, b3 = split(p.astype(np.float64))
    r = lambda a: bf16(np.asarray(a, dtype=np.float32)).astype(np.float64)
    n = len(T)
    Z1 = r(X) @ r(W1) + b1
    H1 = silu(Z1)
    Z2 = r(H1) @ r(W2) + b2
    H2 = silu(Z2)
    y = H2 @ w3 + b3
    res = y - T
    dy = 2.0 * res / n
    dZ2 = dy[:, None] * w3[None, :] * dsilu(Z2)
    g = np.zeros(NP)
    g[192:4288] = (r(H1).T @ r(dZ2)).ravel()
    g[4288:4352] = r(dZ2).sum(0)
    g[4352:4416] = r(H2).T @ r(dy)
    g[4416] = r(dy).sum()
    dH1 = r(dZ2) @ r(W2).T
    dZ1 = dH1 * dsilu(Z1)
    g[0:128] = (r(X).T @ r(dZ1)).ravel()
    g[128:192] = r(dZ1).sum(0)
    return g, float(np.mean(res ** 2))


@pytest.mark.gpu
def test_gradients_match_numpy(gpu_lib):
    rng = np.random.default_rng(5)
    n = 777
    p = np.zeros(NP, dtype=np.float32)
    p[0:128] = rng.standard_normal(128) * 0.17
    p[128:192] = rng.standard_normal(64) * 0.1
    p[192:4288] = rng.standard_normal(4096) * 0.125
    p[4288:4352] = rng.standard_normal(64) * 0.1
    p[4352:4416] = rng.standard_normal(64) * 0.17
    p[4416] = 0.3
    X = rng.uniform(-1, 1, (n, 2)).astype(np.float32)
    T = rng.uniform(0, 1, n).astype(np.float32)
    g = np.zeros(NP, dtype=np.float32)
    loss = C.c_double()
    rc = gpu_lib.trekis_mlp_grad(p.ctypes.data, n, X.ctypes.data, T.ctypes.data, g.ctypes.data, C.byref(loss))
    assert rc == 0, gpu_lib.trekis_last_error()
    ref, ref_loss = reference_grad(p, X.astype(np.float64), T.astype(np.float64))
    assert loss.value == pytest.approx(ref_loss, rel=1e-3)
    for name, sl in (("W1", slice(0, 128)), ("b1", slice(128, 192)), ("W2", slice(192, 4288)),
                     ("b2", slice(4288, 4352)), ("w3", slice(4352, 4416)), ("b3", slice(4416, 4417))):
        a, b = g[sl].astype(np.float64), ref[sl]
        rel = np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30)
        assert rel < 1e-2, (name, rel)


@pytest.fixture(scope="module")
def trained(gpu_lib):
    w = configs.small(configs.cfg1, NMC=4, Tim=30.0)
    for atom in w.material.atoms:
        for sh in atom.shells:
            if sh.designator < 63:
                sh.Radiat = sh.Auger * 2.0
    t = api.Tables(w, lib=gpu_lib)
    rep = api.train_proposal(t, n_samples=10_000_000, epochs=3, batch=8192, E_lo=1.0, E_hi=1e5,
                             n_eval_E=64, n_eval_u=1024)
    return w, t, rep


@pytest.mark.gpu
def test_training_report(trained):
    w, t, rep = trained
    assert rep["n_nets"] >= 4, rep
    assert rep["loss_last"] < 0.1 * rep["loss_first"], rep
    assert 0.05 < rep["accept_rate"] <= 1.0, rep
    # what the network gains: its guess is fewer brackets from the answer than
    # a bisection of the same rows takes probes
    assert rep["mean_walk"] < rep["mean_bisect"], rep
    assert np.isfinite(rep["kl_mean"]) and rep["kl_mean"] >= 0.0, rep


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [1, 0])
def test_proposal_draws_are_exact(trained, precision):
    w, t, _ = trained
    a, sa = api.mc_run(t, api.RunOptions(precision=precision, seed=31, sampler=0))
    b, sb = api.mc_run(t, api.RunOptions(precision=precision, seed=31, sampler=1))
    for f in ("n_events", "n_el_inelastic", "n_el_elastic", "n_hole_events", "n_auger", "n_radiative",
              "n_photon_abs", "n_particles"):
        assert getattr(sa, f) == getattr(sb, f), f
    assert sa.n_el_inelastic > 0
    for k in a.a:
        assert np.array_equal(a[k], b[k]), k

"""CPU checks of the rank predictor's oracle and of the label / policy
bookkeeping (no GPU)."""
import numpy as np

from oracle import mlp as omlp


def test_mlp_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.standard_normal(omlp.N_PARAMS) * 0.2
    X = rng.standard_normal((37, 8))
    T = rng.standard_normal((37, 2))
    loss, g = omlp.loss_and_grad(p, X, T)
    assert abs(loss - 0.5 * np.sum((omlp.forward(p, X) - T) ** 2) / 37) < 1e-12
    idx = rng.choice(omlp.N_PARAMS, 40, replace=False)
    for i in idx:
        e = np.zeros_like(p)
        e[i] = 1e-6
        fd = (omlp.loss_and_grad(p + e, X, T)[0] - omlp.loss_and_grad(p - e, X, T)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_mlp_pack_round_trip():
    rng = np.random.default_rng(1)
    p = rng.standard_normal(omlp.N_PARAMS)
    Ws, bs = omlp.unpack(p)
    assert [W.shape for W in Ws] == [(64, 8), (64, 64), (64, 64), (2, 64)]
    assert np.array_equal(omlp.pack(Ws, bs), p)
    assert omlp.N_PARAMS == 9026


def test_oversampling_label_and_policy_outcome():
    from xped_gb300.learn import oversampling_label, policy_outcome
    s = np.array([1.0, 0.5, 0.3, 0.2, 0.05, 0.01, 0.001])
    assert oversampling_label(s, 2, 7) == 2        # width 4: first unseen s[4] = 0.05 <= 0.1 * s[1]
    assert oversampling_label(s, 0, 7) == 1
    assert oversampling_label(s, 6, 7) == 1        # reaches min(rows, cols)
    rec = dict(dir=0, sectors=[0, 1], keep=np.array([2, 5]), kmin=np.array([40, 40]),
               spectrum=[s, np.linspace(1, 0.1, 40)], features=np.ones((2, 8), np.float32))
    out = policy_outcome([rec], [[6, 5]])
    assert out == dict(columns=11, saturated=1, under_resolved=0, sketched=2, exact_columns=0)
    out = policy_outcome([rec], [[4, 0]])
    assert out == dict(columns=4, saturated=0, under_resolved=0, sketched=1, exact_columns=40)
    out = policy_outcome([rec], [[3, 0]])
    assert out == dict(columns=3, saturated=0, under_resolved=1, sketched=1, exact_columns=40)

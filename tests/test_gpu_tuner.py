"""GPU: the cost model's kernels against the FP64 reference, its training,
and the learned planner against exhaustive measured search."""
import numpy as np
import pytest

from gfft_gb300 import tuner

pytestmark = pytest.mark.gpu


def test_mlp_forward_and_gradients_match_reference(cuda):
    from oracle import mlp_ref
    m = tuner.MLP(nin=24, width=64, depth=3, seed=7)
    p = m.params()
    rng = np.random.default_rng(1)
    X = rng.normal(size=(500, 24)).astype(np.float32)
    y = rng.normal(size=500).astype(np.float32)
    pred = m.predict(X)
    ref = mlp_ref.forward(p, X, 24, 64, 3)
    assert np.max(np.abs(pred - ref)) <= 1e-4 * max(1.0, np.max(np.abs(ref)))
    g, loss = m.gradients(X, y)
    gr = mlp_ref.gradients(p, X, y, 24, 64, 3)
    rel = np.linalg.norm(g - gr) / np.linalg.norm(gr)
    assert rel <= 1e-4, rel
    assert abs(loss - np.mean((ref - y) ** 2)) <= 1e-4 * max(1.0, loss)


def test_mlp_training_fits_smooth_target(cuda):
    rng = np.random.default_rng(2)
    m = tuner.MLP(seed=3)
    X = rng.uniform(-1, 1, size=(1500, m.nin)).astype(np.float32)
    y = (np.sin(2 * X[:, 0]) + 0.5 * X[:, 1] * X[:, 2]).astype(np.float32)
    l0 = float(np.mean((m.predict(X) - y) ** 2))
    l1 = m.train(X, y, epochs=1500, lr=3e-3)
    assert l1 < 0.1 * l0 and l1 < 0.02, (l0, l1)


def test_learned_planner_regret(cuda):
    """What the trained network gains.  Train on measured plans of some
    lengths; for held-out lengths, measure only the model's top 5 candidates
    (the pruned search) and compare with the exhaustive measured search (the
    bar: within 5 % on average) and with the same pruning driven by the
    untrained network; the library's measured choice (`tuner.choose`) adds
    the planner's default plan to the measured set, so it is never worse
    than the default."""
    rng = np.random.default_rng(5)
    pool = [n for n in (2 ** a * 3 ** b * 5 ** c for a in range(4, 19) for b in range(0, 4) for c in range(0, 3))
            if 256 <= n <= 1 << 20]
    pool = sorted(set(pool))
    sizes = rng.choice(pool, 60, replace=False)
    train_sizes, test_sizes = sizes[:44], sizes[44:]
    rows = tuner.timing_table(train_sizes, batch_points=1 << 20, reps=3)
    X = np.array([r["features"] for r in rows], dtype=np.float32)
    ms = np.array([r["ms"] for r in rows], dtype=np.float32)
    model = tuner.CostModel(seed=11)
    loss = model.fit(X, ms, epochs=2500, groups=[r["n"] for r in rows])
    assert loss < 0.5
    untrained = tuner.CostModel(seed=11)
    untrained.mu, untrained.sd = model.mu, model.sd
    k = 5
    top_trained, top_untrained, default, frac, first, with_default = [], [], [], [], [], []
    for n in test_sizes:
        n = int(n)
        b = max(1, (1 << 20) // n)
        cands = tuner.candidates(n, 1, 0, 1, b)
        t = tuner.measure(n, 1, 0, 1, b, cands, reps=5)
        t = np.where(t > 0, t, np.inf)
        best = float(np.min(t))
        Xc = np.stack([tuner.features(n, 1, 0, 1, b, c) for c in cands])
        order = np.argsort(model.predict_ms(Xc))
        top_trained.append(float(np.min(t[order[:k]])) / best - 1)
        first.append(float(t[order[0]]) / best - 1)
        top_untrained.append(float(np.min(t[np.argsort(untrained.predict_ms(Xc))[:k]])) / best - 1)
        default.append(float(t[cands.index({})]) / best - 1)
        with_default.append(min(top_trained[-1], default[-1]))
        frac.append(min(k, len(cands)) / len(cands))
    m_tr, m_un, m_df = float(np.mean(top_trained)), float(np.mean(top_untrained)), float(np.mean(default))
    print("pruned top-%d regret: trained %.3f, untrained %.3f; model's first choice %.3f; default plan %.3f; "
          "measured %.2f of the candidates" % (k, m_tr, m_un, float(np.mean(first)), m_df, float(np.mean(frac))))
    assert m_tr <= 0.05
    assert float(np.mean(with_default)) <= min(m_tr, m_df) + 1e-12
    assert m_tr < m_un
    assert float(np.mean(frac)) <= 0.4


def test_shipped_cost_model_prunes(cuda):
    """The cost model shipped with the package loads and drives a pruned
    search (the best measured of its top 5) to a valid plan."""
    model = tuner.default_model()
    assert model is not None
    opts, ms = tuner.choose(model, 3 * 2 ** 18, 1, 0, 1, 8, k=5)
    assert ms > 0 and isinstance(opts, dict)


def test_learned_plan_choice_in_the_facade(cuda, oracle):
    """TransformObject(plan="learned") takes the shipped cost model's first
    choice, plan="measured" the best measured of its top 5; both transform
    correctly (exact oracle, FP32 bound)."""
    import numpy as np
    from gfft_gb300 import gfft as G
    from gfft_gb300 import inputs
    for plan in ("learned", "measured"):
        for n, b in ((3 * 2 ** 14, 4), (1 << 20, 1), (5 ** 6, 3)):
            obj = G.TransformObject(n, G.FLOAT, G.DFT, 1, G.Serial, G.OUT_OF_PLACE, b, plan=plan)
            x = inputs.gaussian(n + b, 2 * n * b).astype(np.float32)
            xt = cuda.from_numpy(x).cuda()
            y = cuda.empty_like(xt)
            obj.fft(xt, y)
            cuda.cuda.synchronize()
            ex = oracle.fft_ld(x.astype(np.float64), n, b, 1)
            got = y.cpu().numpy().astype(np.float64)
            assert np.linalg.norm(got - ex) / np.linalg.norm(ex) <= 6e-7 * np.log2(n), (plan, n)
            obj.close()

"""The learned eddy-viscosity closure on the GPU against its CPU oracle (oracle/closure.py):
training-data features and targets, network forward and gradient, training, the closure step,
and what a trained network gains over none (held-out samples)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def oc():
    import oracle.closure as m

    return m


def rand_net(rng):
    m = oc()
    theta = rng.normal(0, 0.3, m.NPARAM)
    return theta, rng.normal(0, 1, m.NIN), rng.uniform(0.5, 2.0, m.NIN)


def test_gradient_matches_oracle(ark):
    m = oc()
    rng = np.random.default_rng(7)
    theta, mu, sd = rand_net(rng)
    n = 1000  # several tiles, a ragged last one
    X = (rng.normal(0, 1, (n, m.NIN)) * sd + mu).astype(np.float32)
    t = rng.uniform(0, 3, n).astype(np.float32)
    with ark.ClosureData(4096) as d, ark.Mlp(seed=3) as net:
        d.append(X, t)
        net.set(theta, mu, sd)
        loss, g = net.gradient(d)
        # the oracle on the same BF16-rounded weights and FP32 inputs, FP64 arithmetic
        wq = m.bf16(theta)
        mu32, sd32 = np.float32(mu).astype(np.float64), 1.0 / np.float32(1.0 / sd).astype(np.float64)
        lo, go = m.loss_and_grad(wq, mu32, sd32, X.astype(np.float64), t.astype(np.float64))
        assert abs(loss - lo) <= 2e-5 * lo
        assert np.linalg.norm(g - go) <= 2e-4 * np.linalg.norm(go)
        p = net.predict(d)
        assert np.allclose(p, m.forward(wq, mu32, sd32, X.astype(np.float64)), rtol=2e-4, atol=2e-5)


def test_dataset_features_and_targets_match_oracle(ark, port):
    m = oc()
    p = port.channel_params(16, 12, 8, re_b=2000.0, seed=4, amp=0.15)
    gp = ark.make_params(16, 12, 8, vis=p["nu"], sound=p["sound"], rho0=p["rho0"], cfl=p["cfl"], lx=p["lx"],
                         ly=p["ly"], lz=p["lz"], ub=p["ub"])
    with ark.Context(gp) as c, ark.ClosureData(1 << 16) as d:
        c.upload(port.channel_state(p))
        c.step(3)
        c.sync()
        c.closure_sample(d, sx=1, sz=1, u_tau=0.05)
        assert len(d) == 16 * 12 * 8
        F, T = d.get()
        u = [port.interior(n, c.get(n)) for n in ("u1nCon", "u2nCon", "u3nCon")]
        dx = (p["lx"] / 16, p["ly"] / 12, p["lz"] / 8)
        tgt, ub = m.target(u, dx, p["nu"])
        feat = m.features(ub, dx, p["ly"], 0.05, p["nu"])
        Fo = feat.reshape(-1, m.NIN)
        scale = np.abs(Fo).max(axis=0) + 1e-12
        assert np.all(np.abs(F - Fo) <= 1e-4 * scale + 2e-3 * np.abs(Fo)), np.abs(F - Fo).max(axis=0)
        To = tgt.ravel()
        assert np.allclose(T, To, rtol=2e-3, atol=2e-3 * np.abs(To).max())
        # a lattice subsample takes the rows it names
        c.closure_sample(d, sx=4, sz=2, ox=1, oz=1, u_tau=0.05)
        F2, _ = d.get(16 * 12 * 8)
        sub = feat[1::2, :, 1::4, :].reshape(-1, m.NIN)
        assert np.all(np.abs(F2 - sub) <= 1e-4 * scale + 2e-3 * np.abs(sub))


def test_training_learns_a_teacher(ark):
    """Targets from a fixed teacher network: training lowers the error by a large factor."""
    m = oc()
    rng = np.random.default_rng(11)
    teacher, mu, sd = rand_net(rng)
    X = (rng.normal(0, 1, (1 << 15, m.NIN)) * sd + mu).astype(np.float32)
    t = m.forward(teacher, mu, sd, X.astype(np.float64)).astype(np.float32)
    with ark.ClosureData(1 << 15) as d, ark.Mlp(seed=9) as net:
        d.append(X, t)
        net.fit_normalization(d)
        l0, _ = net.gradient(d)
        l1 = net.train(d, epochs=30, batch=1024, lr=3e-3)
        l2, _ = net.gradient(d)
        assert l2 < 0.05 * l0, (l0, l1, l2)


def test_zero_network_closure_step_is_the_plain_step(ark, port):
    """nu_t = 0 exactly (softplus of a very negative output underflows): the closure step
    equals the plain FP32 step bit for bit, and the closure array is zero."""
    m = oc()
    p = port.channel_params(20, 12, 10, seed=6)
    gp = ark.make_params(20, 12, 10, vis=p["nu"], sound=p["sound"], rho0=p["rho0"], cfl=p["cfl"], lx=p["lx"],
                         ly=p["ly"], lz=p["lz"], ub=p["ub"], precision=ark.FP32)
    theta = np.zeros(m.NPARAM)
    theta[-1] = -200.0
    with ark.Mlp() as net, ark.Context(gp) as a, ark.Context(gp) as b:
        net.set(theta, np.zeros(m.NIN), np.ones(m.NIN))
        st = port.channel_state(p)
        a.upload(st)
        b.upload(st)
        b.set_closure(net, u_tau=0.05)
        a.step(5)
        b.step(5)
        a.sync()
        b.sync()
        names = ["u1nCon", "u2nCon", "u3nCon", "ronCon", "p1", "u11"]
        ra, rb = a.download(names), b.download(names)
        for n in names:
            assert np.array_equal(ra[n].view(np.uint64), rb[n].view(np.uint64)), n
        assert not np.any(b.get("nut"))


def test_closure_changes_the_flow_and_fp64_is_refused(ark, port):
    m = oc()
    p = port.channel_params(20, 12, 10, seed=6)
    base = dict(vis=p["nu"], sound=p["sound"], rho0=p["rho0"], cfl=p["cfl"], lx=p["lx"], ly=p["ly"], lz=p["lz"],
                ub=p["ub"])
    theta = np.zeros(m.NPARAM)
    theta[-1] = 2.0  # nu_t = softplus(2) nu everywhere in the fluid
    with ark.Mlp() as net, ark.Context(ark.make_params(20, 12, 10, precision=ark.FP32, **base)) as c:
        net.set(theta, np.zeros(m.NIN), np.ones(m.NIN))
        c.upload(port.channel_state(p))
        c.set_closure(net, u_tau=0.05)
        c.step(2)
        c.sync()
        nut = c.get("nut")
        inner = port.interior("u1nCon", nut)
        assert np.allclose(inner, np.log1p(np.exp(2.0)) * p["nu"], rtol=1e-6)
        with ark.Context(ark.make_params(20, 12, 10, **base)) as c64:
            with pytest.raises(ark.ArkError) as e:
                c64.set_closure(net, u_tau=0.05)
            assert e.value.status == 6


def test_closure_step_in_both_phase2_forms(ark, port, monkeypatch):
    """The closure's branch (nu_t beside dt and the ghost fill) joins before the stress; the rest
    of the step may run as separate kernels or as the one-kernel Phase2 + second Phase1: the same
    bits either way, with a network that makes nu_t vary from cell to cell."""
    m = oc()
    p = port.channel_params(40, 12, 10, seed=6)
    gp = ark.make_params(40, 12, 10, vis=p["nu"], sound=p["sound"], rho0=p["rho0"], cfl=p["cfl"], lx=p["lx"],
                         ly=p["ly"], lz=p["lz"], ub=p["ub"], precision=ark.FP32)
    theta = np.random.default_rng(3).normal(0.0, 0.3, m.NPARAM)
    names = ["u1nCon", "u2nCon", "u3nCon", "ronCon", "p1", "u11", "p2", "u32", "nut"]
    got = []
    with ark.Mlp() as net:
        net.set(theta, np.zeros(m.NIN), np.ones(m.NIN))
        for form in ("0", "2"):
            monkeypatch.setenv("ARK_PHASE2_FUSED", form)
            with ark.Context(gp) as c:
                c.upload(port.channel_state(p))
                c.set_closure(net, u_tau=0.05)
                c.step(4)
                c.sync()
                got.append(c.download(names[:-1]))
                got[-1]["nut"] = c.get("nut")
    assert np.any(got[0]["nut"])
    for n in names:  # interior cells and computed faces (ghost cells are each form's scratch)
        a = got[0][n] if n == "nut" else port.interior(n, got[0][n])
        b = got[1][n] if n == "nut" else port.interior(n, got[1][n])
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), n


def test_trained_network_beats_no_closure_on_held_out_samples(ark, port):
    """A-priori: trained on the filtered fields of one perturbed channel, the network predicts
    the eddy viscosity of another (held out) with a smaller error than no closure (nu_t = 0)
    or the best constant nu_t."""
    def snapshot(seed, d):
        p = port.channel_params(48, 32, 32, re_b=5600.0, seed=seed, amp=0.3)
        gp = ark.make_params(48, 32, 32, vis=p["nu"], sound=p["sound"], rho0=p["rho0"], cfl=p["cfl"], lx=p["lx"],
                             ly=p["ly"], lz=p["lz"], ub=p["ub"], precision=ark.FP32)
        with ark.Context(gp) as c:
            c.upload(port.channel_state(p))
            c.step(40)
            c.sync()
            c.closure_sample(d, sx=1, sz=1, u_tau=0.032)

    with ark.ClosureData(1 << 17) as train, ark.ClosureData(1 << 17) as test, ark.Mlp(seed=2) as net:
        snapshot(101, train)
        snapshot(202, test)
        net.fit_normalization(train)
        net.train(train, epochs=40, batch=2048, lr=2e-3)
        _, t = test.get()
        pred = net.predict(test)
        mse_net = float(np.mean((pred - t) ** 2))
        mse_zero = float(np.mean(t ** 2))
        _, ttrain = train.get()
        mse_const = float(np.mean((np.mean(ttrain) - t) ** 2))
        assert mse_net < 0.9 * mse_const < 0.9 * mse_zero, (mse_net, mse_const, mse_zero)


def test_tensor_core_inference_matches_oracle(ark):
    """The step's inference (hidden layers as BF16 tensor-core multiplies, FP32 accumulation,
    GELU with the hardware tanh) against the FP64 network: BF16 activations bound the error."""
    m = oc()
    rng = np.random.default_rng(17)
    theta, mu, sd = rand_net(rng)
    n = 5000  # a ragged last warp
    X = (rng.normal(0, 1, (n, m.NIN)) * sd + mu).astype(np.float32)
    with ark.ClosureData(n) as d, ark.Mlp() as net:
        d.append(X, np.zeros(n, np.float32))
        net.set(theta, mu, sd)
        wq = m.bf16(theta)
        mu32, sd32 = np.float32(mu).astype(np.float64), 1.0 / np.float32(1.0 / sd).astype(np.float64)
        want = m.forward(wq, mu32, sd32, X.astype(np.float64))
        tc = net.predict(d, tensor_cores=True)
        fp32 = net.predict(d)
        assert np.allclose(fp32, want, rtol=2e-4, atol=2e-5)
        err = np.abs(tc - want)
        assert np.all(err <= 0.03 * np.abs(want) + 0.02 * np.mean(np.abs(want))), err.max()
        assert np.mean(err) <= 0.01 * np.mean(np.abs(want))

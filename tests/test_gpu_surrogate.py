"""The learned surrogate on the GPU: features bit-exact against the oracle,
network forward pass and gradients against the CPU restatement
(oracle/mlp_oracle.py) within BF16 tolerance, training on plain-solver
trajectories, the ablation against the frame without the network, and the
plain fallback gate."""
import numpy as np
import pytest

from oracle import mlp_oracle as M
from tests.helpers import same_bits

pytestmark = pytest.mark.gpu


def _torch():
    return pytest.importorskip("torch")


def _sim(W, dims, capacity, iterations=4):
    cfg = W.WrachConfig(dimensions=dims, cell_size=1, mode=1, iterations=iterations, gravity=0.1,
                        capacity=capacity)
    return W.Simulation(cfg)


def test_features_match_oracle(W):
    torch = _torch()
    rng = np.random.default_rng(0)
    dims = (60.0, 40.0)
    pos = rng.uniform((0, 0), dims, size=(1500, 2)).astype(np.float32)
    pos[:120] = (20.0 + rng.uniform(-1.2, 1.2, (120, 2))).astype(np.float32)  # over-full cells
    vel = rng.normal(0, 0.7, size=pos.shape).astype(np.float32)
    with _sim(W, dims, 4000) as sim:
        sim.add_particles(pos, vel)
        sim.surrogate_init(0, 16)
        p, v, table = sim.read_frame()
        n = len(p)
        x = torch.zeros((n, 64), dtype=torch.int16, device="cuda")
        sim.surrogate_features(x.data_ptr(), n)
        sim.sync()
        got = x.cpu().numpy().view(np.uint16)
        s = sim.settings()
        want = M.bf16_bits(M.features(s.grid_dimensions[0], s.grid_dimensions[1], 9, table, p, v))
        assert np.array_equal(got, want.astype(np.uint16))


def _random_net(rng, scale=0.25):
    p = rng.normal(0, scale, M.N_PARAMS).astype(np.float32)
    w1, b1, w2, b2, w3, b3 = M.unpack(p)
    w3[:, 2:] = 0.0
    b3[2:] = 0.0
    return M.pack(w1, b1, w2, b2, w3, b3)


def test_forward_and_gradients_match_oracle(W):
    torch = _torch()
    rng = np.random.default_rng(1)
    with _sim(W, (30.0, 30.0), 100) as sim:
        sim.surrogate_init(0, 16)
        params = _random_net(rng)
        sim.surrogate_set_params(params)
        assert np.array_equal(sim.surrogate_params(), params)
        n = 333
        x = M.bf16(rng.normal(0, 0.7, (n, 64)).astype(np.float32))
        t = rng.normal(0, 0.3, (n, 2)).astype(np.float32)
        dx = torch.from_numpy((M.bf16_bits(x).astype(np.uint16)).view(np.int16)).cuda()
        dt = torch.from_numpy(t).cuda()
        dy = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
        y_cpu, _ = M.forward(params, x)
        for kernel in ("tcgen05", "mma"):
            dy.zero_()
            sim.surrogate_forward(dx.data_ptr(), n, dy.data_ptr(), kernel=kernel)
            sim.sync()
            y_gpu = dy.cpu().numpy()
            # BF16 activations: an FP32 vs float64 accumulation can flip an
            # activation's BF16 rounding, one BF16 ulp (2^-8 relative)
            assert np.abs(y_gpu - y_cpu).max() <= 2e-2 * np.abs(y_cpu).max(), kernel
        assert sim.flags() == 0
        g_gpu, l_gpu = sim.surrogate_gradients(dx.data_ptr(), dt.data_ptr(), n)
        g_cpu, l_cpu = M.gradients(params, x, t)
        assert abs(l_gpu - l_cpu) <= 1e-2 * l_cpu
        for name, a, b in zip(("w1", "b1", "w2", "b2", "w3", "b3"), M.unpack(g_gpu), M.unpack(g_cpu)):
            err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
            assert err < 3e-2, (name, err)


@pytest.mark.parametrize("n", [1, 127, 128, 129, 70001, 400009])
def test_tcgen05_forward_matches_mma_forward(W, n):
    # the tcgen05 kernel (tiles of 128 rows in two slots per CTA, accumulators
    # in tensor memory) against the mma.sync kernel on the same rows, ragged
    # last tiles included; 400,009 rows give every CTA several tiles, so both
    # slots and their refills run
    torch = _torch()
    rng = np.random.default_rng(7 + n)
    with _sim(W, (30.0, 30.0), 100) as sim:
        sim.surrogate_init(0, 16)
        sim.surrogate_set_params(_random_net(rng))
        x = M.bf16(rng.normal(0, 0.7, (n, 64)).astype(np.float32))
        dx = torch.from_numpy((M.bf16_bits(x).astype(np.uint16)).view(np.int16)).cuda()
        ya = torch.full((n + 1, 2), 7.0, dtype=torch.float32, device="cuda")
        yb = torch.full((n + 1, 2), 7.0, dtype=torch.float32, device="cuda")
        sim.surrogate_forward(dx.data_ptr(), n, ya.data_ptr(), kernel="tcgen05")
        sim.surrogate_forward(dx.data_ptr(), n, yb.data_ptr(), kernel="mma")
        sim.sync()
        a, b = ya.cpu().numpy(), yb.cpu().numpy()
        assert np.all(a[n] == 7.0)  # nothing written past the rows
        assert np.abs(a[:n] - b[:n]).max() <= 2e-2 * max(np.abs(b[:n]).max(), 1e-3)
        assert sim.flags() == 0


def test_training_beats_the_frame_without_the_network(W):
    # the ablation: trained on plain-solver frames, the network's correction
    # is closer to the plain solver's first three iterations than the zero
    # correction of the frame without it
    from wrach_gb300 import workloads
    dims, pos, vel = workloads.lattice(n=15000, width=240.0, height=136.0, sites=(167, 95))
    with _sim(W, dims, 40000) as sim:
        sim.add_particles(pos, vel)
        sim.surrogate_init(0, 15000 * 40)
        for _ in range(40):
            sim.surrogate_collect()
            sim.step(1)
        first = sim.surrogate_train(1, 4096, 2e-3)
        last = sim.surrogate_train(600, 4096, 2e-3)
        assert last < first
        ratios = []
        for _ in range(5):
            net, zero = sim.surrogate_evaluate()
            ratios.append(net / zero)
            sim.step(1)
        print("held-out frames: mse(network) / mse(no network) =", np.round(ratios, 3))
        assert np.mean(ratios) < 0.7


def test_collect_takes_every_stride_th_taking_part_particle(W):
    rng = np.random.default_rng(6)
    dims = (50.0, 40.0)
    pos = rng.uniform((0, 0), dims, size=(2500, 2)).astype(np.float32)
    pos[:150] = (25.0 + rng.uniform(-1.0, 1.0, (150, 2))).astype(np.float32)  # over-full cells
    vel = rng.normal(0, 0.7, size=pos.shape).astype(np.float32)
    with _sim(W, dims, 4000) as sim:
        sim.add_particles(pos, vel)
        sim.surrogate_init(0, 100000)
        p, v, table = sim.read_frame()
        start = np.asarray(table, np.int64)[1:]
        ntp = int(np.minimum(np.diff(start), 9).sum())
        assert ntp < len(p)
        # call 0: offset 0, stride 1; call 1: offset 1, stride 7
        assert sim.surrogate_collect() == ntp
        assert sim.surrogate_collect(stride=7) == ntp + (ntp - 1 + 6) // 7


def test_fallback_gate(W):
    from wrach_gb300 import workloads
    dims, pos, vel = workloads.lattice(n=12000, width=200.0, height=120.0, sites=(139, 87))
    with _sim(W, dims, 30000) as sur, _sim(W, dims, 30000) as plain:
        sur.add_particles(pos, vel)
        plain.add_particles(pos, vel)
        sur.surrogate_init(3, 16)
        # a bound nothing can meet: frame 0 is a plain calibration frame and
        # every other frame falls back to the plain solve, so the run must
        # equal plain frames bit for bit
        st = sur.surrogate_step(40, max_penetration=-1.0, max_energy_drift=1e9)
        plain.step(40)
        assert st["frames"] == 40 and st["calibrations"] == 2 and st["fallbacks"] == 38
        a, b = sur.read_frame(), plain.read_frame()
        assert np.array_equal(a[2], b[2]) and same_bits(a[0], b[0]) and same_bits(a[1], b[1])
        # the reference overlap is the plain frames' own measure
        assert st["reference_penetration"] > 0.0
        # a bound nothing exceeds: no fallback, and a consistent frame
        st = sur.surrogate_step(6, max_penetration=1e9, max_energy_drift=1e9)
        assert st["frames"] == 6 and st["calibrations"] == 1 and st["fallbacks"] == 0
        p, v, t = sur.read_frame()
        assert int(t[-1]) == len(pos) and np.all(np.diff(t.astype(np.int64)) >= 0)
        assert st["max_energy_drift"] < 0.01


def test_fused_correction_matches_the_separate_kernels(W):
    # the fused kernel of surrogate frames (features in shared memory, the
    # network, the correction) against features -> network through global
    # memory; zero for particles that do not take part
    torch = _torch()
    rng = np.random.default_rng(4)
    dims = (90.0, 50.0)
    pos = rng.uniform((0, 0), dims, size=(3000, 2)).astype(np.float32)
    pos[:200] = (30.0 + rng.uniform(-1.5, 1.5, (200, 2))).astype(np.float32)  # over-full cells
    vel = rng.normal(0, 0.7, size=pos.shape).astype(np.float32)
    with _sim(W, dims, 8000) as sim:
        sim.add_particles(pos, vel)
        sim.surrogate_init(0, 16)
        sim.surrogate_set_params(_random_net(rng))
        p, v, table = sim.read_frame()
        n = len(p)
        x = torch.zeros((n, 64), dtype=torch.int16, device="cuda")
        y = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
        c = torch.full((n, 2), 7.0, dtype=torch.float32, device="cuda")
        sim.surrogate_features(x.data_ptr(), n)
        # the fused pass runs the mma.sync network: the same products in the
        # same order as that forward kernel
        sim.surrogate_forward(x.data_ptr(), n, y.data_ptr(), kernel="mma")
        sim.surrogate_correction(c.data_ptr())
        sim.sync()
        start = np.asarray(table, np.int64)[1:]
        cells = np.repeat(np.arange(len(start) - 1), np.diff(start))
        takes = (np.arange(n) - start[cells]) < 9
        assert 0 < takes.sum() < n
        want = np.where(takes[:, None], y.cpu().numpy(), 0.0)
        got = c.cpu().numpy()
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)


def test_frame_metrics_match_numpy(W):
    rng = np.random.default_rng(5)
    dims = (40.0, 30.0)
    pos = rng.uniform((0, 0), dims, size=(1400, 2)).astype(np.float32)
    pos[:100] = (12.0 + rng.uniform(-1.0, 1.0, (100, 2))).astype(np.float32)
    vel = rng.normal(0, 0.7, size=pos.shape).astype(np.float32)
    with _sim(W, dims, 4000) as sim:
        sim.add_particles(pos, vel)
        mean, mx, ke = sim.frame_metrics()
        p, v, table = sim.read_frame()
        s = sim.settings()
        gx, gy = s.grid_dimensions
    start = np.asarray(table, np.int64)[1:]
    pens = []
    for c in range(gx * gy):
        cy, cx = divmod(c, gx)
        cand = []
        for ny in range(max(cy - 1, 0), min(cy + 1, gy - 1) + 1):
            for nx in range(max(cx - 1, 0), min(cx + 1, gx - 1) + 1):
                js, je = start[ny * gx + nx], start[ny * gx + nx + 1]
                cand.extend(range(js, min(je, js + 9)))
        cand = np.asarray(cand, np.int64)
        for i in range(start[c], min(start[c + 1], start[c] + 9)):
            j = cand[cand != i]
            d = np.sqrt(((p[j] - p[i]).astype(np.float64) ** 2).sum(1))
            pens.append(max(0.0, (1.0 - d).max()) if len(j) else 0.0)
    pens = np.asarray(pens)
    assert abs(mean - pens.mean()) <= 1e-5 * max(pens.mean(), 1e-3)
    assert abs(mx - pens.max()) <= 1e-6
    assert abs(ke - 0.5 * (v.astype(np.float64) ** 2).sum()) <= 1e-5 * ke


def test_surrogate_frames_hold_the_error_bounds(W):
    """Trained on plain frames of a reduced lattice (60,000 particles at the
    1M lattice's density), 320 gated surrogate frames (the configured gate:
    fallback past 0.2 px of excess overlap or 1% of energy drift) stay within
    the error bounds against 320 plain frames from the same state: averaged
    over the last 160 frames (sampled every 32), the mean overlap at most
    0.05 px above the plain frames' and the kinetic energy within 1%."""
    from wrach_gb300 import workloads
    dims, pos, vel = workloads.lattice(n=60000, width=480.0, height=272.0, sites=(334, 188))
    with _sim(W, dims, 120000) as sur, _sim(W, dims, 120000) as plain:
        sur.add_particles(pos, vel)
        plain.add_particles(pos, vel)
        sur.surrogate_init(0, 60000 * 64)
        for f in range(320):
            if f % 5 == 0:
                sur.surrogate_collect()
            sur.step(1)
        sur.surrogate_train(1500, 8192, 2e-3)
        sur.set_particles(pos, vel)
        ms, mp, drift = [], [], 0.0
        for chunk in range(10):
            # chunks of 32 frames: one plain calibration frame and 31 gated
            # surrogate frames each, as one continuous run would have them
            st = sur.surrogate_step(32, max_penetration=0.2, max_energy_drift=0.01)
            plain.step(32)
            drift = max(drift, st["max_energy_drift"])
            ms.append(sur.frame_metrics())
            mp.append(plain.frame_metrics())
    ms, mp = np.array(ms[5:]), np.array(mp[5:])
    print("overlap %s vs %s px; kinetic energy %s vs %s; max drift %.4f"
          % (np.round(ms[:, 0], 4), np.round(mp[:, 0], 4), np.round(ms[:, 2], 0),
             np.round(mp[:, 2], 0), drift))
    assert drift <= 0.01
    assert ms[:, 0].mean() - mp[:, 0].mean() <= 0.05
    assert abs(ms[:, 2].mean() / mp[:, 2].mean() - 1.0) <= 0.01

"""GPU parity of batched uneven-length complex transforms (work list, CUDA graph, per-transform loop)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_uneven_batch_matches_oracle(engine, oracle_lib, dtype):
    from impulse_gb300 import _lib as L
    from impulse_gb300.batch import MultiFFT, uneven_lengths
    lengths = uneven_lengths(count=400, total=1 << 22, lo=2, hi=1 << 17, seed=11)
    lengths += [1, 2, 3, 8191, 16384, 32768, 65537 if dtype == "f32" else 40000]
    code = L.IG_F32 if dtype == "f32" else L.IG_F64
    tdt = torch.complex64 if dtype == "f32" else torch.complex128
    rng = np.random.default_rng(4)
    tot = sum(lengths)
    x = (rng.standard_normal(tot) + 1j * rng.standard_normal(tot))
    X = torch.from_numpy(x).to("cuda", dtype=tdt)
    plan = MultiFFT(lengths, code, forward=True, fct=0.5)
    assert plan.info["worklist"] > 0 and plan.info["fourstep"] > 0 and plan.info["general"] > 0
    s = torch.cuda.Stream()
    outs = {}
    with torch.cuda.stream(s):
        for mode in ("worklist", "graph", "loop"):
            Y = torch.zeros_like(X)
            plan.run(X.data_ptr(), Y.data_ptr(), s.cuda_stream, mode)
            if mode == "graph":  # replay
                Y.zero_()
                plan.run(X.data_ptr(), Y.data_ptr(), s.cuda_stream, mode)
            s.synchronize()
            outs[mode] = Y.cpu().numpy()
    pos = 0
    for n in lengths:
        seg = x[pos:pos + n]
        want = oracle_lib.cfft(seg, True, 0.5)
        tol = 1e-12 if dtype == "f64" else 1e-6 * max(1.0, np.log2(n)) * 2
        for mode, y in outs.items():
            got = y[pos:pos + n]
            assert oracle_lib.rel_l2(got, want) < tol, (mode, n, oracle_lib.rel_l2(got, want))
        pos += n


def test_uneven_offsets_and_inplace(engine, oracle_lib):
    from impulse_gb300 import _lib as L
    from impulse_gb300.batch import MultiFFT
    lengths = [5, 16, 16, 100, 4096, 9000, 7, 16]
    offsets, pos = [], 3
    for n in lengths:
        offsets.append(pos)
        pos += n + 5  # gaps between transforms
    rng = np.random.default_rng(9)
    x = rng.standard_normal(pos) + 1j * rng.standard_normal(pos)
    X = torch.from_numpy(x).cuda()
    plan = MultiFFT(lengths, L.IG_F64, forward=False, fct=1.0, offsets=offsets)
    plan.run(X.data_ptr(), X.data_ptr(), None, "worklist")  # in place
    torch.cuda.synchronize()
    y = X.cpu().numpy()
    for n, o in zip(lengths, offsets):
        assert oracle_lib.rel_l2(y[o:o + n], oracle_lib.cfft(x[o:o + n], False)) < 1e-12
    mask = np.ones(pos, bool)
    for n, o in zip(lengths, offsets):
        mask[o:o + n] = False
    assert np.array_equal(y[mask], x[mask])

"""Training the learned indicator through the C ABI alone: the C++ driver
(host/train_indicator.cpp, built as _build/wenofd_train) uses only
wenofd_create / wenofd_advance / wenofd_indicator_sample / wenofd_mlp_init /
wenofd_mlp_train, with no Python or PyTorch.  Two runs with the same seed give
the same parameters bit for bit, and so does the Python workflow
(wenofd.learned) with the same settings."""
import os
import subprocess

import numpy as np
import pytest

import wenofd
from conftest import ROOT

pytestmark = pytest.mark.gpu

TRAINER = os.path.join(ROOT, "fd-weno-eulerequation_gb300", "_build", "wenofd_train")
SMALL = dict(n=128, snapshots=(10, 30), per_snapshot=12_000, epochs=3, batch=1024, seed=5)


def _train_cabi(path):
    args = [TRAINER, path, "--n", str(SMALL["n"]), "--snapshots", ",".join(map(str, SMALL["snapshots"])),
            "--per-snapshot", str(SMALL["per_snapshot"]), "--epochs", str(SMALL["epochs"]), "--batch",
            str(SMALL["batch"]), "--seed", str(SMALL["seed"])]
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    p = np.fromfile(path, dtype=np.float32)
    assert p.size == wenofd.MLP_PARAMS
    return p, r.stdout


def test_c_abi_training_is_repeatable_and_matches_the_python_workflow(tmp_path):
    a, out = _train_cabi(str(tmp_path / "a.bin"))
    b, _ = _train_cabi(str(tmp_path / "b.bin"))
    assert np.array_equal(a, b)
    print("\n" + out.strip())
    torch = pytest.importorskip("torch")
    from wenofd import learned

    X, y = learned.generate_dataset(torch, n=SMALL["n"], snapshots=SMALL["snapshots"],
                                    per_snapshot=SMALL["per_snapshot"])
    # about half of each snapshot's sample is flagged (both classes exist here)
    frac = float(y.mean())
    assert 0.3 < frac < 0.7
    assert abs(len(y) - 4 * 2 * SMALL["per_snapshot"]) < 0.05 * 4 * 2 * SMALL["per_snapshot"]
    p, _ = learned.train(torch, X, y, epochs=SMALL["epochs"], batch=SMALL["batch"], lr=3e-3, seed=SMALL["seed"])
    assert np.array_equal(p, a)


def test_sampler_is_seeded_and_balanced():
    torch = pytest.importorskip("torch")
    cfg = {"TESTCASE": 5, "ELEMNUMX": 160, "ELEMNUMY": 160, "RKMETH": 2, "CFL": 0.7, "SCHEME": 1, "SEED": 3,
           "PRECISION": wenofd.FP32}
    with wenofd.Solver(cfg) as s:
        s.initialize()
        s.advance(max_steps=20)
        n = 160 * 160
        feat = torch.empty((n, 50), dtype=torch.float32, device="cuda")
        lab = torch.empty(n, dtype=torch.uint8, device="cuda")
        s.indicator_data(feat.data_ptr(), lab.data_ptr())
        cap = 6000
        X1 = torch.empty((cap, 50), dtype=torch.float32, device="cuda")
        y1 = torch.empty(cap, dtype=torch.float32, device="cuda")
        X2, y2 = torch.empty_like(X1), torch.empty_like(y1)
        r1 = s.indicator_sample(4000, 99, X1.data_ptr(), y1.data_ptr(), cap)
        r2 = s.indicator_sample(4000, 99, X2.data_ptr(), y2.data_ptr(), cap)
        r3 = s.indicator_sample(4000, 100, X2.data_ptr(), y2.data_ptr(), cap)
        torch.cuda.synchronize()
    npos = int(lab.sum())
    assert r1 == r2 and abs(r1 - 4000) < 300 and r3 > 0
    m = min(r1, r3)
    assert not torch.equal(X1[:m], X2[:m])  # another seed keeps other cells
    k = y1[:r1].cpu().numpy()
    want_pos = min(npos, 2000)
    assert abs(k.sum() - want_pos) < 0.15 * want_pos + 50
    # every sampled row is the feature row of some node with that label
    F = feat.cpu().numpy()
    L = lab.cpu().numpy()
    rows = X1[:r1].cpu().numpy()
    index = {}
    for i in range(n):
        index.setdefault(F[i].tobytes(), set()).add(int(L[i]))
    for r in range(0, r1, 37):
        assert int(k[r]) in index[rows[r].tobytes()]

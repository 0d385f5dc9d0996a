"""Training workflow of the learned troubled-cell indicator.

Data come from the solver itself: shear-layer (or Riemann) runs at seeds other
than the evaluation seed; at several times, every cell's 50 features and its
WENO-Z label are extracted on the GPU (wenofd_indicator_data) and a balanced
sample is kept.  Training runs the project's FP32 forward / backward / Adam
kernels (wenofd_mlp_train).  torch supplies device buffers only.
"""
from __future__ import annotations

import numpy as np

from . import FP32, MLP_INPUTS, MLP_PARAMS, Solver, mlp_forward, mlp_train


def init_params(seed: int) -> np.ndarray:
    """Uniform He-style initialisation (same layout as the C ABI)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(MLP_PARAMS, dtype=np.float32)
    p[0:1600] = rng.uniform(-1, 1, 1600) * np.sqrt(6.0 / 50)
    p[1632:2656] = rng.uniform(-1, 1, 1024) * np.sqrt(6.0 / 32)
    p[2688:2720] = rng.uniform(-1, 1, 32) * np.sqrt(6.0 / 32)
    return p


DEFAULT_RUNS = ((5, 11), (5, 12), (4, 13), (4, 14))


def generate_dataset(torch, runs=DEFAULT_RUNS, n: int = 512, snapshots=(40, 120, 240, 400),
                     per_snapshot: int = 125_000, device: int = 0, sample_seed: int = 0,
                     label_deviation: float = 1e-2):
    """Features X (N, 50) and labels y (N,) as CUDA float32 tensors: for each
    (testcase, seed) run, an FP32-form solve at n x n, and at each snapshot
    step a sample of `per_snapshot` cells, half flagged and half not where
    possible.  Defaults: two shear layers and two seeded Riemann problems,
    4 x 4 x 125k = 2e6 stencils."""
    gen = torch.Generator(device=f"cuda:{device}")
    gen.manual_seed(sample_seed)
    Xs, ys = [], []
    cells = n * n
    feat = torch.empty((cells, MLP_INPUTS), dtype=torch.float32, device=f"cuda:{device}")
    lab = torch.empty(cells, dtype=torch.uint8, device=f"cuda:{device}")
    for testcase, seed in runs:
        with Solver({"TESTCASE": testcase, "ELEMNUMX": n, "ELEMNUMY": n, "RKMETH": 2, "CFL": 0.7, "SCHEME": 1,
                     "SEED": seed, "PRECISION": FP32, "DEVICE": device, "TEND": 1.0e9,
                     "LABEL_DEVIATION": label_deviation}) as s:
            s.initialize()
            done = 0
            for snap in snapshots:
                s.advance(max_steps=snap - done)
                done = snap
                s.indicator_data(feat.data_ptr(), lab.data_ptr())
                torch.cuda.synchronize(device)
                pos = torch.nonzero(lab, as_tuple=True)[0]
                neg = torch.nonzero(lab == 0, as_tuple=True)[0]
                k_pos = min(len(pos), per_snapshot // 2)
                k_neg = min(len(neg), per_snapshot - k_pos)
                pick = []
                if k_pos:
                    pick.append(pos[torch.randperm(len(pos), generator=gen, device=pos.device)[:k_pos]])
                if k_neg:
                    pick.append(neg[torch.randperm(len(neg), generator=gen, device=neg.device)[:k_neg]])
                idx = torch.cat(pick)
                Xs.append(feat[idx].clone())
                ys.append(lab[idx].float())
    X = torch.cat(Xs)
    y = torch.cat(ys)
    perm = torch.randperm(len(y), generator=gen, device=y.device)
    return X[perm].contiguous(), y[perm].contiguous()


def train(torch, X, y, epochs: int = 20, batch: int = 4096, lr: float = 3e-3, seed: int = 1,
          init_seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """Train on the GPU with the project's kernels; returns (params, epoch losses)."""
    params = torch.from_numpy(init_params(init_seed)).to(X.device)
    stream = torch.cuda.current_stream(X.device).cuda_stream
    losses = mlp_train(params.data_ptr(), X.data_ptr(), y.data_ptr(), len(y), epochs, batch, lr, seed, stream)
    return params.cpu().numpy(), losses


def predict_logits(torch, params: np.ndarray, X):
    p = torch.from_numpy(np.ascontiguousarray(params, dtype=np.float32)).to(X.device)
    out = torch.empty(len(X), dtype=torch.float32, device=X.device)
    mlp_forward(p.data_ptr(), X.data_ptr(), len(X), out.data_ptr(), torch.cuda.current_stream(X.device).cuda_stream)
    return out


def recall_precision(torch, params: np.ndarray, X, y, threshold: float = 0.5) -> tuple[float, float, float]:
    """Recall and precision of the flags on (X, y), and the flagged fraction."""
    logits = predict_logits(torch, params, X)
    flag = logits > float(np.log(threshold / (1 - threshold)))
    yb = y > 0.5
    tp = (flag & yb).sum().item()
    recall = tp / max(1, yb.sum().item())
    precision = tp / max(1, flag.sum().item())
    return recall, precision, flag.float().mean().item()

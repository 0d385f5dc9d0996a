"""Training workflow of the learned troubled-cell indicator.

Data come from the solver itself: shear-layer (or Riemann) runs at seeds other
than the evaluation seed; at several times a balanced sample of cells, their
50 features and WENO-Z labels, is formed on the GPU (wenofd_indicator_sample).
Training runs the project's FP32 forward / backward / Adam kernels
(wenofd_mlp_train) from wenofd_mlp_init's parameters.  torch supplies device
buffers only; the same steps through the C ABI alone are
fd-weno-eulerequation_gb300/host/train_indicator.cpp, which gives the same
parameters bit for bit.
"""
from __future__ import annotations

import numpy as np

from . import FP32, MLP_INPUTS, Solver, mlp_forward, mlp_init, mlp_train


def init_params(seed: int) -> np.ndarray:
    """Uniform He-style initialisation (wenofd_mlp_init)."""
    return mlp_init(seed)


DEFAULT_RUNS = ((5, 11), (5, 12), (4, 13), (4, 14))


def sample_seed_of(sample_seed: int, run: int, snapshot: int) -> int:
    """Seed of the device sampler for one snapshot of one run."""
    return (sample_seed * 1_000_003 + run * 1_009 + snapshot) & 0xFFFFFFFFFFFFFFFF


def generate_dataset(torch, runs=DEFAULT_RUNS, n: int = 512, snapshots=(40, 120, 240, 400),
                     per_snapshot: int = 125_000, device: int = 0, sample_seed: int = 0,
                     label_deviation: float = 1e-2):
    """Features X (N, 50) and labels y (N,) as CUDA float32 tensors: for each
    (testcase, seed) run, an FP32-form solve at n x n, and at each snapshot
    step a device-side sample of about `per_snapshot` cells, half flagged and
    half not where possible (wenofd_indicator_sample), appended in order.
    Defaults: two shear layers and two seeded Riemann problems, 4 x 4 x 125k
    = 2e6 stencils."""
    slack = 1.05
    cap = int(len(runs) * len(snapshots) * (per_snapshot * slack + 1024))
    X = torch.empty((cap, MLP_INPUTS), dtype=torch.float32, device=f"cuda:{device}")
    y = torch.empty(cap, dtype=torch.float32, device=f"cuda:{device}")
    rows = 0
    for r, (testcase, seed) in enumerate(runs):
        with Solver({"TESTCASE": testcase, "ELEMNUMX": n, "ELEMNUMY": n, "RKMETH": 2, "CFL": 0.7, "SCHEME": 1,
                     "SEED": seed, "PRECISION": FP32, "DEVICE": device, "TEND": 1.0e9,
                     "LABEL_DEVIATION": label_deviation}) as s:
            s.initialize()
            done = 0
            for k, snap in enumerate(snapshots):
                s.advance(max_steps=snap - done)
                done = snap
                rows += s.indicator_sample(per_snapshot, sample_seed_of(sample_seed, r, k), X[rows:].data_ptr(),
                                           y[rows:].data_ptr(), cap - rows)
    torch.cuda.synchronize(device)
    return X[:rows].contiguous(), y[:rows].contiguous()


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

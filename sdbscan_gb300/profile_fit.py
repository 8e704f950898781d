"""One fit_sDbscan on the config-2 law at a chosen size, with the engine's
per-stage CUDA-event times and counters printed.  Small enough to run under
a profiler:

    python -m sdbscan_gb300.profile_fit N [precision] [d]

precision 0 = plain FP32 (default), 1 = BF16 screening.
"""
import sys


def main(argv):
    import torch

    from sdbscan_gb300 import capi, datasets
    n = int(argv[1]) if len(argv) > 1 else 100_000
    prec = int(argv[2]) if len(argv) > 2 else 0
    d = int(argv[3]) if len(argv) > 3 else 784
    X, _ = datasets.cfg2_mnist_like_torch(n, d, seed=2007, device="cuda")
    torch.cuda.synchronize()
    eng = capi.Engine(n, d)
    eng.set_params(n_proj=1024, topK=10, topM=50, distance="Cosine", random_seed=42, precision=prec)
    eng.fit_sdbscan_device(X.data_ptr(), 0.25, 50)
    print(eng.stage_ms(), eng.counters())


if __name__ == "__main__":
    main(sys.argv)

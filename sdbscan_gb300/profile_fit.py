"""One fit_sDbscan on the config-2 law at a chosen size, with the engine's
per-stage CUDA-event times and counters printed.  Small enough to run under
a profiler:

    python -m sdbscan_gb300.profile_fit N [precision] [d] [distance]

precision 0 = plain FP32 (default), 1 = BF16 mode; distance Cosine (default),
L1 or L2 (random-Fourier embedding, ker 1024, sigma 1) or Chi2.
"""
import sys


def main(argv):
    import torch

    from sdbscan_gb300 import capi, datasets
    n = int(argv[1]) if len(argv) > 1 else 100_000
    prec = int(argv[2]) if len(argv) > 2 else 0
    d = int(argv[3]) if len(argv) > 3 else 784
    dist = argv[4] if len(argv) > 4 else "Cosine"
    X, _ = datasets.cfg2_mnist_like_torch(n, d, seed=2007, device="cuda")
    torch.cuda.synchronize()
    eng = capi.Engine(n, d)
    kw = dict(ker_n_features=1024, ker_sigma=1.0) if dist in ("L1", "L2", "Chi2", "JS") else {}
    eng.set_params(n_proj=1024, topK=10, topM=50, distance=dist, random_seed=42, precision=prec, **kw)
    eng.fit_sdbscan_device(X.data_ptr(), 0.25, 50)
    print(eng.stage_ms(), eng.counters())


if __name__ == "__main__":
    main(sys.argv)

"""One fit_sngDbscan on the config-2 law (d = 784) at a chosen size, with the
engine's per-stage CUDA-event times and counters printed.  Small enough to
run under a profiler:

    python -m sdbscan_gb300.profile_sng N [precision] [samplingProb]

precision 0 = plain FP32 (default), 1 = BF16 screening; samplingProb 0.01
(default); eps 0.25, minPts 50, seed 42.
"""
import sys


def main(argv):
    import torch

    from sdbscan_gb300 import capi, datasets
    n = int(argv[1]) if len(argv) > 1 else 200_000
    prec = int(argv[2]) if len(argv) > 2 else 0
    prob = float(argv[3]) if len(argv) > 3 else 0.01
    X, _ = datasets.cfg2_mnist_like_torch(n, 784, seed=2007, device="cuda")
    torch.cuda.synchronize()
    eng = capi.Engine(n, 784)
    eng.set_sng_params(distance="Cosine", samplingProb=prob, random_seed=42)
    eng.set_precision(prec)
    eng.fit_sngdbscan_device(X.data_ptr(), 0.25, 50)
    print(eng.stage_ms(), eng.counters())


if __name__ == "__main__":
    main(sys.argv)

"""Train the far-field surrogate on seeded synthetic networks and save a checkpoint.

    python ddd.jl_gb300/train_surrogate.py --config gpu65k --seeds 11 12 13 14 \
        --pairs 2500000 --epochs 20 --out ddd.jl_gb300/data/surrogate_gpu65k_nu028.bin

Every step runs on the GPU through the library: pair sampling picks far pairs
(R >= 0.9 kappa max(L_i, L_j)) of each network, the FP64 kernel computes their
exact forces (ddd_surrogate_make_data), the tcgen05 training kernels fit the
network (ddd_surrogate_train, Adam, cosine decay), and the checkpoint records the
parameters with kappa, the Poisson ratio and the core radius it was trained for.
The networks come from the same generator as the benchmark workloads
(synth.py) with seeds other than the benchmark's seed 0, so the benchmark
network is never seen in training.
"""
import argparse
import importlib.util
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))


def _package():
    if "ddd_gb300" in sys.modules:
        return sys.modules["ddd_gb300"]
    spec = importlib.util.spec_from_file_location("ddd_gb300", os.path.join(HERE, "__init__.py"),
                                                  submodule_search_locations=[HERE])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["ddd_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def train(config="gpu65k", seeds=(11, 12, 13, 14), pairs=2500000, epochs=20, batch=4096, lr=2e-3, kappa=20.0,
          out=None, seed=5, device=0):
    pkg = _package()
    import ddd_gb300.synth as synth
    ctx = pkg.get_context(device)
    k = pkg.consts_of(pkg.DislocationParameters(coreRad=synth.CORE_RAD), pkg.MaterialParameters(mu=synth.MU,
                                                                                                  nu=synth.NU))
    nets = []
    for s in seeds:
        p, b, _ = synth.make(config, seed=s)
        nets.append(synth.packed_soa(p, b))
    sur = pkg.Surrogate(ctx, seed=seed)
    t0 = time.time()
    info = sur.fit(k, nets, pairs_per_network=pairs, epochs=epochs, batch=batch, lr=lr, kappa=kappa, seed=seed)
    info["seconds"] = time.time() - t0
    if out:
        os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
        sur.save(out)
    return sur, info


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="gpu65k")
    ap.add_argument("--seeds", type=int, nargs="+", default=[11, 12, 13, 14])
    ap.add_argument("--pairs", type=int, default=2500000, help="training pairs per network (4 x 2.5e6 = 1e7)")
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--kappa", type=float, default=20.0)
    ap.add_argument("--out", required=True)
    a = ap.parse_args()
    _, info = train(a.config, a.seeds, a.pairs, a.epochs, a.batch, a.lr, a.kappa, a.out)
    print(json.dumps({"out": a.out, "samples": info["samples"], "seconds": info["seconds"],
                      "loss_first": float(info["loss"][0]), "loss_last": float(info["loss"][-1])}))


if __name__ == "__main__":
    main()

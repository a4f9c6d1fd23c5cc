"""Train the learned preconditioner on the GPU and write its weights.

    python -m ouranos_gb300.train_preconditioner [--n 64] [--maps 128] [--fields 4]
        [--epochs 8] [--pairs synthetic|solver|dsa-guess] [--out ouranos_gb300/weights/precond_thick3d.npz]

The committed weights ouranos_gb300/weights/dsa_guess_thick3d.npz come from

    python -m ouranos_gb300.train_preconditioner --pairs dsa-guess --n 32 --maps 512 \\
        --fields 16 --passes 2 --epochs 8 --out ouranos_gb300/weights/dsa_guess_thick3d.npz

Training maps are the seeded 3-D thick diffusive material maps (seeds
2000, 2001, ...; GLC S12); evaluation maps use other seeds.  --pairs synthetic
trains on (A e, e) for seeded error fields e; --pairs solver on the Krylov
vectors FGMRES meets, each with its converged diffusion correction as the
target (--fields is then the number of Arnoldi steps per map and pass);
--pairs dsa-guess trains the network as the initial guess of the diffusion
correction's CG (ouranos_rt_pc_dsa_apply) on the Krylov vectors of FGMRES
with that preconditioner, and reports the iterations of the evaluation map
(seed 7000, 64^3) with and without the network for several CG budgets.
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--maps", type=int, default=128)
    ap.add_argument("--fields", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--sn", type=int, default=12)
    ap.add_argument("--pairs", choices=("synthetic", "solver", "dsa-guess"), default="synthetic")
    ap.add_argument("--inner-cg", type=int, default=3, help="dsa-guess: CG steps of the collection solves")
    ap.add_argument("--passes", type=int, default=2, help="solver pairs: collection passes")
    ap.add_argument("--out", default=os.path.join(HERE, "weights", "precond_thick3d.npz"))
    args = ap.parse_args()
    import ouranos_gb300
    ouranos_gb300.build()
    from ouranos_gb300.learned import compare_dsa_guess, train, train_dsa_guess, train_on_solver_pairs
    t0 = time.time()
    log = lambda s: print(s, flush=True)  # noqa: E731
    if args.pairs == "dsa-guess":
        net, hist = train_dsa_guess(n=args.n, maps=args.maps, steps_per_map=args.fields, passes=args.passes,
                                    epochs=args.epochs, lr=args.lr, sn=args.sn, inner_cg=args.inner_cg, log=log)
    elif args.pairs == "solver":
        net, hist = train_on_solver_pairs(n=args.n, maps=args.maps, steps_per_map=args.fields,
                                          passes=args.passes, epochs=args.epochs, lr=args.lr, sn=args.sn,
                                          log=log)
    else:
        net, hist = train(n=args.n, maps=args.maps, fields_per_map=args.fields, epochs=args.epochs,
                          lr=args.lr, sn=args.sn, log=log)
    dt = time.time() - t0
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    net.save(args.out, meta={"loss_history": hist, "maps": args.maps, "fields": args.fields,
                             "epochs": args.epochs, "train_seconds": dt, "n": args.n, "pairs": args.pairs})
    print(json.dumps({"trained": args.out, "seconds": dt, "final_loss": hist[-1]}), flush=True)
    if args.pairs == "dsa-guess":
        print(json.dumps({"evaluation_seed7000_64cubed": compare_dsa_guess(args.out)}), flush=True)


if __name__ == "__main__":
    main()

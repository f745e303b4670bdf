"""Offline autotuner for the launch shapes of the CUDA-core gradient and the step kernel.

Two knobs decide how a fit's work is cut into launches, both set through
the library's gbnuts_set_launch_shape(split_rows_min, team_warps):

  split_rows_min  minimum rows per split of the CUDA-core partial kernel
                  (fp64 / fp32 forms; splits are also bounded by about two
                  waves of CTAs over the device's SMs and, for the
                  hierarchical families, by the group count)
  team_warps      warps per chain of the step kernel (1, 2, 4 or 8; by
                  default 1 up to D = 64, 2 up to 1024, 8 above)

The setting is process-wide, so each candidate runs in its own process: a
short adaptive fit of the workload, timed with CUDA events (device ms per
step).  The tuner prints the table and the best candidate and can write them
as JSON.  The library's built-in rules were set from such sweeps; the knobs
exist so a deployment can re-tune for its own shapes.  A fit's row splits
determine the order of its gradient sums, so a tuned setting changes the draws
at round-off level (results stay deterministic for a fixed setting).

    python -m stan_gb300.autotune --workload hier_normal --chains 256 --precision fp32
"""
import argparse
import itertools
import json
import os
import subprocess
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)

SPLIT_ROWS = (64, 128, 256, 512, 1024)
TEAM_WARPS = (1, 2, 4, 8)


def _candidate(args):
    """Runs in the child process: one short fit, prints its timing as JSON."""
    from stan_gb300 import Model, _lib, sampler, workloads
    _lib.check(_lib.load().gbnuts_set_launch_shape(args.split_rows, args.team_warps),
               "gbnuts_set_launch_shape")
    ds = workloads.make_dataset(args.workload, seed=1)
    m = Model.from_dataset(ds)
    kw = dict(num_chains=args.chains, num_warmup=args.iters, num_samples=0,
              precision=args.precision, random_seed=1, max_depth=10)
    sampler.run(m, **dict(kw, num_warmup=max(4, args.iters // 4)))  # warm-up run
    r = sampler.run(m, **kw)
    print(json.dumps({"ms_per_step": r.total_ms / r.steps, "grad_ms": r.grad_ms,
                      "steps": int(r.steps)}))


def sweep(workload, chains, precision, iters=30, split_rows=SPLIT_ROWS, team_warps=TEAM_WARPS,
          python=sys.executable, timeout=600):
    """Times every (split_rows, team_warps) candidate; returns (rows, best)."""
    rows = []
    for sr, tw in itertools.product(split_rows, team_warps):
        cmd = [python, "-m", "stan_gb300.autotune", "--child", "--workload", workload,
               "--chains", str(chains), "--precision", precision, "--iters", str(iters),
               "--split-rows", str(sr), "--team-warps", str(tw)]
        r = subprocess.run(cmd, cwd=_ROOT, capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            rows.append({"split_rows": sr, "team_warps": tw, "error": r.stderr[-300:]})
            continue
        res = json.loads(r.stdout.strip().splitlines()[-1])
        rows.append({"split_rows": sr, "team_warps": tw, **res})
    ok = [x for x in rows if "ms_per_step" in x]
    best = min(ok, key=lambda x: x["ms_per_step"]) if ok else None
    return rows, best


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--workload", default="hier_normal")
    ap.add_argument("--chains", type=int, default=256)
    ap.add_argument("--precision", default="fp32", choices=["fp64", "fp32", "bf16x3", "f16x3"])
    ap.add_argument("--iters", type=int, default=30)
    ap.add_argument("--split-rows", default=",".join(map(str, SPLIT_ROWS)))
    ap.add_argument("--team-warps", default=",".join(map(str, TEAM_WARPS)))
    ap.add_argument("--out", default=None, help="write the table and the best as JSON")
    ap.add_argument("--child", action="store_true", help=argparse.SUPPRESS)
    args = ap.parse_args(argv)
    if args.child:
        args.split_rows = int(args.split_rows)
        args.team_warps = int(args.team_warps)
        _candidate(args)
        return
    rows, best = sweep(args.workload, args.chains, args.precision, args.iters,
                       tuple(int(v) for v in args.split_rows.split(",")),
                       tuple(int(v) for v in args.team_warps.split(",")))
    for x in rows:
        print(json.dumps(x))
    result = {"workload": args.workload, "chains": args.chains, "precision": args.precision,
              "iters": args.iters, "candidates": rows, "best": best}
    print(json.dumps({"best": best}))
    if args.out:
        with open(args.out, "w") as f:
            json.dump(result, f, indent=1)


if __name__ == "__main__":
    main()

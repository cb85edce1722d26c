"""Step one of the benchmark workloads a fixed number of times (command-line
counterpart of the reference's script action Advance, src/scripts.rs:334-337).

    python physics-sim_gb300/run_steps.py --workload c1_chains --steps 80
"""
import argparse
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import dem  # noqa: E402
import dem_scenes  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="c1_chains")
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--particles", type=int, default=0, help="particles (dense_bed) or scenes (c3_batch)")
    ap.add_argument("--graph-steps", type=int, default=35)
    ap.add_argument("--plain", action="store_true", help="no CUDA graphs (for ncu)")
    ap.add_argument("--split", action="store_true", help="Simulation pass as k_narrow + k_forces")
    ap.add_argument("--unfused", action="store_true", help="every step its own LOM kernel")
    ap.add_argument("--cell-factor", type=float, default=0.0, help="search_cell_factor (0: default)")
    ap.add_argument("--skin", type=float, default=0.0, help="list_skin (0: default)")
    ap.add_argument("--block", type=int, default=0, help="block_size (0: default)")
    a = ap.parse_args()
    knobs = {"split_narrow": int(a.split), "unfused_lom": int(a.unfused), "search_cell_factor": a.cell_factor,
             "list_skin": a.skin, "block_size": a.block}
    if a.workload == "c3_batch":
        items = dem_scenes.c3_batch(n_scenes=a.particles or 512)
        with dem.Batch(items, reorder_interval=a.graph_steps, plain_launches=a.plain, **knobs) as b:
            b.step(a.steps)
            b.synchronize()
            print("ok", a.workload, len(items), "scenes", sum(len(x[0]["radii"]) for x in items),
                  "particles", a.steps, "steps", b.stats())
        return
    if a.workload == "c1_chains":
        sc, p, ext = dem_scenes.c1_chains()
    elif a.workload == "c0_settle":
        sc, p, ext = dem_scenes.c0_settle()
    elif a.workload == "c2_impact":
        sc, p, ext = dem_scenes.c2_impact()
    elif a.workload == "dense_bed":
        sc, p, ext = dem_scenes.dense_bed(n=a.particles or (1 << 20))
    else:
        raise SystemExit("unknown workload")
    with dem.Context(sc, p, reorder_interval=a.graph_steps, plain_launches=a.plain, **knobs, **ext) as ctx:
        ctx.step(a.steps)
        ctx.synchronize()
        print("ok", a.workload, len(sc["radii"]), "particles", a.steps, "steps", ctx.stats())


if __name__ == "__main__":
    main()

"""Command line: run a reference-format multigroup deck on the GPU, or write
one of the synthetic problems as a deck.

  python -m abeille_gb300 run DECK.yaml [--precision mixed] [--particles N]
                                        [--generations G] [--ignored I]
                                        [--tracking delta-tracking] [--device D]
  python -m abeille_gb300 write-config {0,1,2} OUT.yaml [--particles N]

`run` follows the deck's settings (simulation, nparticles, ngenerations,
nignored, transport, seed, stride) unless overridden, and prints the results
the reference prints at the end of a run (src/power_iterator.cpp,
src/fixed_source.cpp), plus the device throughput.
"""
import argparse
import sys

from . import deck as _deck
from . import decks
from .engine import Engine


def run_deck(path_or_text, precision="mixed", particles=None, generations=None, ignored=None, tracking=None,
             device=0, out=sys.stdout, is_text=False):
    """Run a deck; returns the run statistics dictionary."""
    kw = {"precision": precision}
    if particles:
        kw["nparticles"] = particles
    if tracking:
        kw["tracking"] = tracking
    builder, d = _deck.deck_from_text(path_or_text, **kw) if is_text else _deck.load_deck(path_or_text, **kw)
    st = d.get("settings", {})
    ngen = int(generations or st.get("ngenerations", 100))
    nign = int(ignored if ignored is not None else st.get("nignored", 0 if builder.mode == "fixed-source" else 10))
    eng = Engine(builder.build(precision=precision), device)
    try:
        if builder.mode != "fixed-source":  # k-eigenvalue, branching or branchless
            stats, recs = eng.run_power_iteration_records(ngen, nign)
            print(f" {'gen':>5} {'k_col':>10} {'entropy':>10}", file=out)
            for i, r in enumerate(recs):
                print(f" {i + 1:5d} {r['kcol']:10.6f} {r['entropy']:10.6f}", file=out)
            print(f"\n k_col    = {stats['kcol_avg']:.6f} +/- {stats['kcol_std']:.6f}", file=out)
            print(f" k_trk    = {stats['ktrk_avg']:.6f} +/- {stats['ktrk_std']:.6f}", file=out)
            print(f" leakage  = {stats['leak_avg']:.6f} +/- {stats['leak_std']:.6f}", file=out)
            print(f" mig area = {stats['mig_avg']:.6f} +/- {stats['mig_std']:.6f}", file=out)
        else:
            stats = eng.run_fixed_source(ngen, builder.nparticles)
            print(f" leakage = {stats['leak_avg']:.6f} +/- {stats['leak_std']:.6f}", file=out)
        secs = stats["transport_ms"] / 1e3
        print(f"\n {stats['collisions']} collisions, {stats['histories']} histories, "
              f"{stats['collisions'] / secs / 1e6 if secs > 0 else 0.0:.1f} M collisions/s in transport "
              f"({precision})", file=out)
        return stats
    finally:
        eng.close()


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m abeille_gb300")
    sub = ap.add_subparsers(dest="cmd", required=True)
    r = sub.add_parser("run", help="run a multigroup deck")
    r.add_argument("deck")
    r.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    r.add_argument("--particles", type=int)
    r.add_argument("--generations", type=int)
    r.add_argument("--ignored", type=int)
    r.add_argument("--tracking", choices=["delta-tracking", "surface-tracking", "implicit-leakage-delta-tracking",
                                             "carter-tracking"])
    r.add_argument("--device", type=int, default=0)
    w = sub.add_parser("write-config", help="write a synthetic problem as a deck")
    w.add_argument("config", type=int, choices=sorted(decks.CONFIGS))
    w.add_argument("out")
    w.add_argument("--particles", type=int)
    a = ap.parse_args(argv)
    if a.cmd == "run":
        run_deck(a.deck, a.precision, a.particles, a.generations, a.ignored, a.tracking, a.device)
        return 0
    b = decks.CONFIGS[a.config](**({"nparticles": a.particles} if a.particles else {}))
    gens = {0: (70, 20), 1: (50, 10), 2: (50, 10)}[a.config]
    with open(a.out, "w") as f:
        f.write(_deck.dump_yaml(b.to_deck(ngenerations=gens[0], nignored=gens[1])) + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())

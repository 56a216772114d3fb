"""Runs of the reference's own multigroup transport code (test
infrastructure: the checker of the oracle).

oracle/refshim/build_ref.py compiles the reference's unmodified sources with
stand-in headers into oracle/_ref/abeille_ref; this module writes a deck (the
dictionary ProblemBuilder.to_deck gives) and a bank to files, runs the driver
and reads back what the reference produced: sampled source banks
(Simulation::sample_sources, src/simulation.cpp:55-77), and the fission bank,
the generation's score sums and mesh-tally arrays of one
Transporter::transport call.
"""
import json
import os
import subprocess
import tempfile

import numpy as np

from . import PARTICLE_DTYPE, SITE_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
SCORES = ("k_col", "k_abs", "k_trk", "leakage", "k_tot", "mig_area")


def driver():
    """Path of the reference driver, built if needed; None where the reference
    tree or pcg-cpp is not available (the reason is printed)."""
    from .refshim import build_ref
    return build_ref.build(quiet=False)


class ReferenceRun:
    def __init__(self, deck, exe=None):
        self.exe = exe or driver()
        if not self.exe:
            raise RuntimeError("the reference driver is not available")
        self.dir = tempfile.mkdtemp(prefix="abeille_ref_")
        self.deck_path = os.path.join(self.dir, "deck.json")
        with open(self.deck_path, "w") as f:
            json.dump(deck, f)
        self.ntally = len(deck.get("tallies", []))

    def _run(self, nsample, bank_path, kcol, converged, out):
        r = subprocess.run([self.exe, self.deck_path, str(nsample), bank_path, repr(float(kcol)),
                            str(int(bool(converged))), out], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference run failed ({r.returncode}): {r.stderr[-2000:]}")

    def sample_sources(self, n):
        out = os.path.join(self.dir, "src")
        self._run(n, "-", 1.0, True, out)
        return np.fromfile(out + ".bank", dtype=PARTICLE_DTYPE)

    def transport(self, bank, kcol=1.0, converged=True):
        """(sites, scores, tallies): the fission bank in the order the
        reference returns it, the raw score sums of the generation, and every
        mesh tally's generation array (collision estimators first)."""
        bank_path = os.path.join(self.dir, "bank.bin")
        np.ascontiguousarray(bank, PARTICLE_DTYPE).tofile(bank_path)
        out = os.path.join(self.dir, "tr")
        self._run(0, bank_path, kcol, converged, out)
        sites = np.fromfile(out + ".sites", dtype=SITE_DTYPE)
        vals = np.loadtxt(out + ".scores")
        tallies = [np.fromfile(f"{out}.tally{i}") for i in range(self.ntally)]
        return sites, dict(zip(SCORES, map(float, vals))), tallies

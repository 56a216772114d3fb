"""The reference-side binding compiles and links inside the reference.

include/abeille_gb300_transporter.hpp (GpuTransporter, a Transporter
subclass) is compiled against the reference's own headers and linked with
the reference's own objects (oracle/refshim/build_ref.py) and
libabeille_gb300.so into oracle/_ref/adapter_check.  The program reads a deck
with the library's native reader and constructs the transporter: on a
machine without a GPU the construction ends in the reference's fatal_error
with the engine's reason (status 1); with a GPU the context is created.
Runs where the reference tree is present; skipped elsewhere.
"""
import json
import os
import subprocess

import pytest

from abeille_gb300 import deck, decks

HERE = os.path.dirname(os.path.abspath(__file__))
DECKS = json.load(open(os.path.join(HERE, "golden", "reference_decks.json")))


@pytest.fixture(scope="module")
def exe():
    from oracle.refshim import build_ref
    path = build_ref.build_adapter_check()
    if not path:
        pytest.skip("the reference cannot be built here")
    return path


@pytest.mark.parametrize("name", ["c5g7", "Ua-1-1-CY", "quadrics"])
def test_gpu_transporter_links_inside_the_reference(exe, name, tmp_path):
    if name == "quadrics":
        d = decks.quadrics(nparticles=100, tracking="surface-tracking").to_deck(ngenerations=5, nignored=1)
    else:
        d = {k: v for k, v in DECKS[name].items() if not k.startswith("_")}
    path = tmp_path / "deck.yaml"
    path.write_text(deck.dump_yaml(d))
    r = subprocess.run([exe, str(path)], capture_output=True, text=True, timeout=120)
    out = r.stdout + r.stderr
    assert f"{len(d['cells'])} cells" in out and f"{len(d['materials'])} materials" in out, out
    if r.returncode == 0:
        assert "context created" in out
    else:
        assert r.returncode == 1 and "GPU transporter:" in out and "CUDA" in out, out

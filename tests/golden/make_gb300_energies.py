"""Record the GB300 model's energies of the bm1_head fixture for the reference driver's validator.

Runs on a GB300 (from the repository root):  python tests/golden/make_gb300_energies.py

For every (PPWI, wgsize) of RUNS it does what the C++ model (minibude_gb300/model/gb300/fasten.hpp)
does in `fasten`: upload the deck, take bude_gpu_default_cfg(PPWI, wgsize), evaluate, download; and
writes the energies as little-endian float32 to tests/golden/bm1_head/gb300/p<PPWI>_w<wgsize>.f32.
tests/test_reference_validator.py replays them through the reference's own driver and checks,
on a GB300, that the model still produces them."""
from __future__ import annotations

import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# PPWI x wgsize combinations the reference driver accepts for 1,024 poses (a multiple of both).
RUNS = [(p, w) for p in (1, 8, 16) for w in (32, 64)]
OUT = os.path.join(HERE, "bm1_head", "gb300")


def model_energies(ctx, deck, ppwi, wgsize):
    """The C++ model's sequence: upload, default launch shape, one evaluation, download."""
    ctx.upload(deck)
    ctx.run(ctx.default_cfg(ppwi, wgsize))
    return ctx.download()


def main() -> None:
    from minibude_gb300 import build, read_deck
    from minibude_gb300.model import GpuContext, device_name
    build.build_library()
    deck = read_deck(os.path.join(HERE, "bm1_head"))
    os.makedirs(OUT, exist_ok=True)
    with GpuContext(0) as ctx:
        for p, w in RUNS:
            model_energies(ctx, deck, p, w).astype("<f4").tofile(os.path.join(OUT, f"p{p}_w{w}.f32"))
    with open(os.path.join(OUT, "source.txt"), "w") as f:
        f.write(f"GB300 model energies of tests/golden/bm1_head ({deck.nposes} poses) recorded on {device_name(0)} by "
                "tests/golden/make_gb300_energies.py: bude_gpu_default_cfg(PPWI, wgsize) for "
                + ", ".join(f"({p}, {w})" for p, w in RUNS) + ".\n")
    print(OUT)


if __name__ == "__main__":
    main()

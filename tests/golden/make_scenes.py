"""Writes the scene fixtures under tests/golden/scenes/ with the reference's
own scene generator (model/python/gen_target_iq.py of
fpga-professional-association/agilex-7-radar-detect): the iq_ascii_v1 sample
file and its ground-truth JSON for each named scenario, medium geometry
(config/medium.json: 4 antennas, 256-point FFT, 2 samples per cycle,
16 frames), seed 1. Run here, where the reference checkout is present:

    python tests/golden/make_scenes.py <reference checkout>
"""
import gzip
import sys
from pathlib import Path

if len(sys.argv) != 2:
    sys.exit("usage: make_scenes.py <reference checkout>")
ref = Path(sys.argv[1])
sys.path.insert(0, str(ref / "model" / "python"))

import gen_target_iq as g  # noqa: E402

OUT = Path(__file__).resolve().parent / "scenes"
OUT.mkdir(exist_ok=True)
cfg = g.load_config(ref / "config" / "medium.json")
for name in ("three_targets", "three_targets_even", "mixed_parity"):
    scen = g.build_scenario(name, cfg, 1)
    re_i, im_i = g.quantise_iq(g.synthesize_iq(scen, cfg))
    iq = g.render_iq(scen, cfg, re_i, im_i)
    with gzip.open(OUT / f"{name}_seed1.iq.gz", "wt", encoding="utf-8", newline="\n") as fh:
        fh.write(iq)
    (OUT / f"{name}_seed1.json").write_text(g.render_json(scen, cfg), encoding="utf-8")
    print(name, len(iq.splitlines()), "lines")

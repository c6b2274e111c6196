"""Writes tests/golden/rvg/<name>.rvg.xz from the reference's shipped scenes.

The reference ships eight RVG scenes (workdir/input/rvg: car, chord,
chord-black, drops, embrace, reschart, test, tiger) that its RVG::load
(VkScanlinePR/src/core/vg/rvg.cpp:9-255) reads.  They are stored here,
xz-compressed and unchanged, so that the parity tests can render them on a
machine without the reference checkout.  The scenes are MIT-licensed by the
reference's author; NOTICE in the same folder carries the notice.

  python tests/golden/make_rvg_fixtures.py <reference>/workdir/input/rvg
"""
import lzma
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "rvg")
NAMES = ["car", "chord", "chord-black", "drops", "embrace", "reschart", "test", "tiger"]


def main(src):
    os.makedirs(OUT, exist_ok=True)
    for n in NAMES:
        with open(os.path.join(src, n + ".rvg"), "rb") as f:
            data = f.read()
        with open(os.path.join(OUT, n + ".rvg.xz"), "wb") as f:
            f.write(lzma.compress(data, preset=9 | lzma.PRESET_EXTREME))
        print("%-12s %8d -> %8d bytes" % (n, len(data), os.path.getsize(os.path.join(OUT, n + ".rvg.xz"))))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    main(sys.argv[1])

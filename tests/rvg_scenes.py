"""The reference's shipped RVG scenes, from the compressed fixtures in
tests/golden/rvg (written by tests/golden/make_rvg_fixtures.py)."""
import lzma
import os

HERE = os.path.dirname(os.path.abspath(__file__))
RVG_DIR = os.path.join(HERE, "golden", "rvg")
NAMES = ["car", "chord", "chord-black", "drops", "embrace", "reschart", "test", "tiger"]


def rvg_text(name):
    with open(os.path.join(RVG_DIR, name + ".rvg.xz"), "rb") as f:
        return lzma.decompress(f.read())


def rvg_file(name, tmpdir):
    """Writes the decompressed scene under tmpdir and returns its path."""
    p = os.path.join(str(tmpdir), name + ".rvg")
    if not os.path.exists(p):
        with open(p, "wb") as f:
            f.write(rvg_text(name))
    return p


def load(sr, name, tmpdir, full=False):
    """(scene dict for scenes.to_oracle/to_container, viewport) of a shipped
    scene, parsed by the library's RVG reader (full: with arcs, quadratics
    and gradients)."""
    sc, vp = sr.load_rvg(rvg_file(name, tmpdir), full=full)
    a = sc.arrays()
    d = dict(width=int(vp[2]), height=int(vp[3]), **a)
    if sc.paints:
        d["paints"] = sc.paints
    return d, vp

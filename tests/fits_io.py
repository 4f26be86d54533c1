"""Minimal HEALPix FITS map files for the tests: one binary table of float32
columns (the layout src/healpix_extra.c:132-164 writes), optionally with rows of
`repeat` elements and NESTED ordering, as other HEALPix writers produce."""
import numpy as np


def _card(text):
    return text.ljust(80)[:80]


def _header(cards):
    raw = "".join(_card(c) for c in cards) + _card("END")
    raw += " " * ((2880 - len(raw) % 2880) % 2880)
    return raw.encode("ascii")


def write_map(path, columns, nside, ordering="RING", repeat=1, names=("T", "Q", "U")):
    cols = [np.asarray(c, np.float32) for c in columns]
    npix = 12 * nside * nside
    assert all(c.size == npix for c in cols) and npix % repeat == 0
    nrows = npix // repeat
    prim = ["SIMPLE  = %20s" % "T", "BITPIX  = %20d" % 8, "NAXIS   = %20d" % 0, "EXTEND  = %20s" % "T"]
    ext = ["XTENSION= 'BINTABLE'", "BITPIX  = %20d" % 8, "NAXIS   = %20d" % 2,
           "NAXIS1  = %20d" % (4 * repeat * len(cols)), "NAXIS2  = %20d" % nrows,
           "PCOUNT  = %20d" % 0, "GCOUNT  = %20d" % 1, "TFIELDS = %20d" % len(cols)]
    for i in range(len(cols)):
        ext += ["TTYPE%-3d= '%-8s'" % (i + 1, names[i]), "TFORM%-3d= '%-8s'" % (i + 1, "%dE" % repeat),
                "TUNIT%-3d= '%-8s'" % (i + 1, "mK")]
    ext += ["PIXTYPE = 'HEALPIX '", "ORDERING= '%-8s'" % ordering, "NSIDE   = %20d" % nside,
            "COORDSYS= 'G       '"]
    rows = np.stack([c.reshape(nrows, repeat) for c in cols], axis=1)  # [row][col][elem]
    data = rows.astype(">f4").tobytes()
    data += b"\0" * ((2880 - len(data) % 2880) % 2880)
    with open(path, "wb") as f:
        f.write(_header(prim) + _header(ext) + data)


def read_map(path, col=0):
    """(header cards of the table, float32 column `col` in file order)"""
    raw = open(path, "rb").read()

    def header(off):
        cards = {}
        while True:
            block = raw[off:off + 2880]
            off += 2880
            for i in range(36):
                c = block[80 * i:80 * i + 80].decode("ascii")
                key = c[:8].strip()
                if key == "END":
                    return cards, off
                if c[8:10] == "= ":
                    cards[key] = c[10:].split("/")[0].strip().strip("'").strip()

    _, off = header(0)
    h, off = header(off)
    nrows, ncols = int(h["NAXIS2"]), int(h["TFIELDS"])
    reps = [int(h["TFORM%d" % (i + 1)][:-1] or 1) for i in range(ncols)]
    assert all(h["TFORM%d" % (i + 1)].endswith("E") for i in range(ncols))
    width = sum(reps)
    tab = np.frombuffer(raw[off:off + 4 * width * nrows], dtype=">f4").reshape(nrows, width)
    start = sum(reps[:col])
    return h, tab[:, start:start + reps[col]].reshape(-1).astype(np.float32)

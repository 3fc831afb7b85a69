"""Generate tests/golden/output/sac_output.npz from the reference's SAC output.

Runs ``oracle/_ref/ref_probe sac`` (the reference's io_recv_output_sac,
io_recv_output_sac_el_iso_strain and io_line_output_sac over lib/sacLib.c,
built by ``make -C oracle``) on seeded station and line seismograms and
stores the inputs together with the bytes of every file it writes.

This script needs the reference build and runs only where it exists; the
fixture it writes is committed and is all the tests need elsewhere.

    python tests/golden/output/make_sac_golden.py
"""

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
PROBE = os.path.join(REPO, "oracle", "_ref", "ref_probe")


def inputs(seed=7, nr=3, ncmp=9, nt=37, nl=2):
    rng = np.random.default_rng(seed)
    names = ["ST%02d" % r for r in range(nr)]
    xyz = rng.uniform(-5e3, 5e3, (nr, 3)).astype(np.float32)
    lam = rng.uniform(2e10, 4e10, nr).astype(np.float32)
    mu = rng.uniform(1e10, 3e10, nr).astype(np.float32)
    amp = np.array([1e-3] * 3 + [1e7] * 6, np.float32)[:, None]
    seismo = (rng.standard_normal((nr, ncmp, nt)) * amp).astype(np.float32)
    lxyz = rng.uniform(-5e3, 5e3, (nl, 3)).astype(np.float32)
    lseq = np.arange(1, nl + 1, dtype=np.int32) * 3
    lseismo = (rng.standard_normal((nl, ncmp, nt)) * amp).astype(np.float32)
    return dict(dt=np.float32(0.0125), evtnm="evt1", names=names, xyz=xyz, lam=lam,
                mu=mu, seismo=seismo, line_name="line2", line_seq=lseq,
                line_xyz=lxyz, line_seismo=lseismo)


def probe_input(d):
    nr, ncmp, nt = d["seismo"].shape
    nl = d["line_seismo"].shape[0]
    b = struct.pack("<4if", nr, ncmp, nt, nl, float(d["dt"]))
    b += d["evtnm"].encode().ljust(16, b"\0")
    for r in range(nr):
        b += d["names"][r].encode().ljust(16, b"\0")
        b += struct.pack("<5f", *d["xyz"][r], d["lam"][r], d["mu"][r])
    b += d["seismo"].astype("<f4").tobytes()
    b += d["line_name"].encode().ljust(16, b"\0")
    for r in range(nl):
        b += struct.pack("<i3f", int(d["line_seq"][r]), *d["line_xyz"][r])
    b += d["line_seismo"].astype("<f4").tobytes()
    return b


def main():
    d = inputs()
    files = {}
    with tempfile.TemporaryDirectory() as tmp:
        inp = os.path.join(tmp, "in.bin")
        with open(inp, "wb") as fh:
            fh.write(probe_input(d))
        out = os.path.join(tmp, "out")
        os.mkdir(out)
        subprocess.run([PROBE, "sac", inp, out], check=True)
        for fn in sorted(os.listdir(out)):
            with open(os.path.join(out, fn), "rb") as fh:
                files["file:" + fn] = np.frombuffer(fh.read(), np.uint8)
    arrays = {k: np.asarray(v) for k, v in d.items()}
    np.savez_compressed(os.path.join(HERE, "sac_output.npz"), **arrays, **files)
    print("wrote %d files' bytes" % len(files))


if __name__ == "__main__":
    main()

"""Generate tests/golden/nersc_4x4x4x4.npz from Chroma's NERSC known-answer fixture.

Source: ``tests/t_asqtad_prop/t_nersc.cfg`` of the Chroma tree (a 4^4 SU(3) archive,
DATATYPE 4D_SU3_GAUGE, IEEE32BIG, whose header records PLAQUETTE and LINK_TRACE).
The npz keeps the parsed header fields and the raw big-endian payload bytes, so the
tests can rebuild an archive byte stream and exercise the oracle's reader and the
12-real reconstruction without the Chroma tree being present.

Usage:  python tests/golden/make_nersc_fixture.py path/to/chroma   (the root of a Chroma source tree)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(chroma_root):
    path = os.path.join(chroma_root, "tests", "t_asqtad_prop", "t_nersc.cfg")
    raw = open(path, "rb").read()
    end = raw.index(b"END_HEADER")
    end = raw.index(b"\n", end) + 1
    header = raw[:end].decode("ascii", "replace")
    fields = {}
    for line in header.splitlines():
        if "=" in line:
            k, v = line.split("=", 1)
            fields[k.strip()] = v.strip()
    dims = [int(fields[f"DIMENSION_{i}"]) for i in range(1, 5)]
    payload = np.frombuffer(raw[end:], dtype=np.uint8)
    out = os.path.join(HERE, "nersc_4x4x4x4.npz")
    np.savez_compressed(out, dims=np.array(dims, dtype=np.int32), payload=payload,
                        plaquette=float(fields["PLAQUETTE"]), link_trace=float(fields["LINK_TRACE"]),
                        datatype=fields["DATATYPE"], floating_point=fields["FLOATING_POINT"],
                        checksum=fields["CHECKSUM"])
    print(out, dims, payload.size, fields["PLAQUETTE"], fields["LINK_TRACE"])


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    main(sys.argv[1])

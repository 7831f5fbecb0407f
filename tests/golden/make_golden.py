"""Generate the golden fixtures used by the parity tests.

Run once in a checkout that has the reference repository available, with
the path of the reference checkout as the argument:

    python tests/golden/make_golden.py REFERENCE_ROOT

It writes three small JSON files next to this script:

* ``reftests.json`` -- the 14 golden arrays of the reference's own test suite
  (``test/reftest-files/*.bson``, produced by ``test/test_1D.jl:21-46``,
  ``test/test_2D.jl:17-53`` and ``test/test_3D_{1..5}.jl``).  Each entry holds
  the 12 sampled cell-centre coordinates ``X`` and the sampled solution ``H``
  (12, 12x12 or 12x12x12 values) flattened in Julia column-major order (x
  fastest), with its ``size``.
* ``iteration_counts.json`` -- the published total PT iteration counts of the
  convergence studies, ``output/out_diff_{1D,2D,3D}_{lin,linstep,nonlin}.txt``
  (rows ``nx [ny [nz]] ittot nt``).
* ``output_rows.json`` -- the first three rows of every ``output/out_*.txt``
  file verbatim (count rows and the perf scripts' timing rows), for the
  byte-exact round trip of the output writer.

The BSON files are read with the small decoder below (BSON 1.0 documents as
written by Julia's BSON.jl: an array is ``{tag:"array", type, size, data}``
with ``data`` the raw little-endian Float64 payload).  Floats are written with
``repr`` so that they round-trip bit-exactly.
"""
import json
import os
import re
import struct
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _cstring(buf, i):
    j = buf.index(b"\x00", i)
    return buf[i:j].decode(), j + 1


def _document(buf, i):
    (length,) = struct.unpack_from("<i", buf, i)
    end = i + length
    i += 4
    out = {}
    while i < end - 1:
        kind = buf[i]
        i += 1
        key, i = _cstring(buf, i)
        if kind == 0x01:
            val = struct.unpack_from("<d", buf, i)[0]
            i += 8
        elif kind == 0x02:
            (n,) = struct.unpack_from("<i", buf, i)
            val = buf[i + 4:i + 4 + n - 1].decode()
            i += 4 + n
        elif kind in (0x03, 0x04):
            val, i = _document(buf, i)
        elif kind == 0x05:
            (n,) = struct.unpack_from("<i", buf, i)
            val = bytes(buf[i + 5:i + 5 + n])
            i += 5 + n
        elif kind == 0x08:
            val = bool(buf[i])
            i += 1
        elif kind == 0x10:
            val = struct.unpack_from("<i", buf, i)[0]
            i += 4
        elif kind == 0x12:
            val = struct.unpack_from("<q", buf, i)[0]
            i += 8
        elif kind == 0x0A:
            val = None
        else:
            raise ValueError(f"unsupported BSON element type {kind:#x}")
        out[key] = val
    return out, end


def _julia_array(node):
    """Decode a BSON.jl Float64 array node into (size, flat column-major list)."""
    assert node["tag"] == "array", node
    assert list(node["type"]["name"].values()) == ["Core", "Float64"], node["type"]
    size = [int(v) for v in node["size"].values()]
    data = node["data"]
    count = 1
    for s in size:
        count *= s
    assert len(data) == 8 * count
    return size, list(struct.unpack(f"<{count}d", data))


def read_reftest(path):
    with open(path, "rb") as fh:
        doc, _ = _document(fh.read(), 0)
    xs, x = _julia_array(doc["X"])
    hs, h = _julia_array(doc["H"])
    return {"X": x, "H": h, "size": hs}


def read_counts(path):
    rows = []
    with open(path) as fh:
        for line in fh:
            if line.strip():
                rows.append([int(v) for v in line.split()])
    return rows


def main(root):
    ref_dir = os.path.join(root, "test", "reftest-files")
    golden = {}
    for name in sorted(os.listdir(ref_dir)):
        if name.endswith(".bson"):
            golden[name[len("test_"):-len(".bson")]] = read_reftest(os.path.join(ref_dir, name))
    with open(os.path.join(HERE, "reftests.json"), "w") as fh:
        fh.write("{\n")
        fh.write(",\n".join(f"{json.dumps(k)}: {json.dumps(v)}" for k, v in golden.items()))
        fh.write("\n}\n")

    counts = {}
    pat = re.compile(r"^out_diff_(1D|2D|3D)_(lin|linstep|nonlin)\.txt$")
    out_dir = os.path.join(root, "output")
    for name in sorted(os.listdir(out_dir)):
        m = pat.match(name)
        if m:
            counts[f"{m.group(1)}_{m.group(2)}"] = read_counts(os.path.join(out_dir, name))
    with open(os.path.join(HERE, "iteration_counts.json"), "w") as fh:
        fh.write("{\n")
        fh.write(",\n".join(f"{json.dumps(k)}: {json.dumps(v)}" for k, v in counts.items()))
        fh.write("\n}\n")
    # the first rows of every output file, verbatim (format round trips)
    rows = {}
    for name in sorted(os.listdir(out_dir)):
        if name.startswith("out_") and name.endswith(".txt"):
            with open(os.path.join(out_dir, name)) as fh:
                rows[name] = [ln.rstrip("\n") for ln in fh if ln.strip()][:3]
    with open(os.path.join(HERE, "output_rows.json"), "w") as fh:
        json.dump(rows, fh, indent=1)
        fh.write("\n")
    print(f"wrote {len(golden)} golden arrays, {len(counts)} iteration-count tables, "
          f"{len(rows)} output-row samples")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])

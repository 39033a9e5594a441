"""The reference engine itself as a checker — TEST INFRASTRUCTURE ONLY.

``oracle/ref.mk`` compiles the reference (SlothDB) from its own sources into
``oracle/_ref/`` and links ``oracle/ref_harness.cpp`` against it.  This
module feeds the harness seeded columns (loaded with the reference's
``Connection::CreateTable`` + ``Connection::Append``) or a Parquet file path,
runs one SQL query through ``Connection::Query`` and parses the result.

It exists only where the reference's sources are (the container that builds
the repository); tests that need it skip elsewhere, and the golden fixtures
it generates are committed under ``tests/golden/``.  Nothing in the product
imports it.
"""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
HARNESS = os.path.join(REF_DIR, "ref_harness")
TYPE_NAMES = {1: "SMALLINT", 2: "INTEGER", 3: "BIGINT", 4: "DOUBLE", 5: "VARCHAR"}
NP = {"SMALLINT": np.int16, "INTEGER": np.int32, "BIGINT": np.int64, "DOUBLE": np.float64}


def reference_source():
    """The reference checkout to build from (None where there is none)."""
    src = os.environ.get("SLOTHDB_REFERENCE_SRC", "/root/reference")
    return src if os.path.isdir(os.path.join(src, "src", "execution")) else None


def build(jobs: int = 0) -> str | None:
    """Build the reference library and the harness (idempotent; make decides
    what is stale).  Returns the harness path, or None without the sources."""
    src = reference_source()
    if src is None:
        return None
    jobs = jobs or os.cpu_count() or 4
    p = subprocess.run(["make", "-f", os.path.join(HERE, "ref.mk"), "REF=" + src, "-j%d" % jobs],
                       capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("reference build failed:\n" + p.stdout[-4000:] + p.stderr[-4000:])
    return HARNESS


def available() -> bool:
    return os.path.exists(HARNESS)


def _parse(path):
    with open(path, "rb") as f:
        header = f.readline().decode().rstrip("\n").split("\t")
        lines = f.read().split(b"\n")
    if lines and lines[-1] == b"":
        lines.pop()
    ncol = len(header)
    cells = [ln.split(b"\t") for ln in lines]
    cols = []
    for c in range(ncol):
        t = header[c]
        raw = [r[c] for r in cells]
        null = np.array([x == b"\\N" for x in raw], dtype=bool)
        if t in ("DOUBLE", "FLOAT"):
            vals = np.array([0.0 if n else float(x) for x, n in zip(raw, null)], dtype=np.float64)
        elif t in ("SMALLINT", "INTEGER", "BIGINT", "HUGEINT"):
            vals = np.array([0 if n else int(x) for x, n in zip(raw, null)], dtype=np.int64)
        else:
            vals = np.array([b"" if n else x for x, n in zip(raw, null)], dtype=object)
        cols.append((t, vals, null))
    return cols


def query(sql, col_types=None, cols=None, names=None, nulls=None, repeat=1):
    """Run `sql` through the reference engine.  cols (optional): numpy arrays
    loaded as table ``t`` (VARCHAR columns: (offsets int64[n+1], bytes)),
    named `names` (default c0, c1, ...).  Returns (columns, median ms) where
    columns is a list of (type name, values, null flags)."""
    if not available():
        raise RuntimeError("reference harness not built (oracle/ref.mk)")
    with tempfile.TemporaryDirectory(prefix="refq_") as d:
        spec = []
        if cols is not None:
            names = names or ["c%d" % i for i in range(len(cols))]
            t0 = TYPE_NAMES[col_types[0]]
            n = len(cols[0][0]) - 1 if t0 == "VARCHAR" else len(cols[0])
            spec.append("rows %d" % n)
            for i, (a, ct) in enumerate(zip(cols, col_types)):
                tn = TYPE_NAMES[ct]
                dp = os.path.join(d, "c%d.bin" % i)
                np_ = "-"
                if nulls is not None and nulls[i] is not None:
                    np_ = os.path.join(d, "c%d.nul" % i)
                    np.asarray(nulls[i], dtype=np.uint8).tofile(np_)
                if tn == "VARCHAR":
                    offs, data = a
                    np.asarray(data, dtype=np.uint8).tofile(dp)
                    op = os.path.join(d, "c%d.off" % i)
                    np.asarray(offs, dtype=np.int64).tofile(op)
                    spec.append("col %s %s %s %s %s" % (names[i], tn, dp, np_, op))
                else:
                    np.ascontiguousarray(a, dtype=NP[tn]).tofile(dp)
                    spec.append("col %s %s %s %s" % (names[i], tn, dp, np_))
        spec.append("repeat %d" % repeat)
        spec.append("query " + sql.replace("\n", " "))
        sp = os.path.join(d, "spec.txt")
        with open(sp, "w") as f:
            f.write("\n".join(spec) + "\n")
        out = os.path.join(d, "out.tsv")
        p = subprocess.run([HARNESS, sp, out], capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("reference query failed (%d): %s" % (p.returncode, p.stderr[-2000:]))
        ms = float([ln.split()[1] for ln in p.stdout.splitlines() if ln.startswith("ms ")][0])
        return _parse(out), ms

"""Generate tests/golden/screening_golden.npz from the reference's own task
partitioner and disjoint set (src/GP/pipeline/partt.py, disjoint_set.py),
loaded from the read-only reference checkout (PW_REFERENCE_DIR, by default a
sibling of this repository named "reference").  Machines without the checkout
read only the file written here.

Contents:
* partition cases (nkey_total, max_chunks, min_chunk_size): the task count of
  partt.guess_chunk_number over np.tril_indices(nkey) and, for three tasks,
  the (from, to) key indices of _partition_screening (solve2.py:78-94) as
  partt.get_task_chunk produces them;
* root-selection cases: random keys' screening edges, disentangled flags and
  scheme bases, and the screened key indices of each scheme, computed with
  the reference's DisjointSet by the loop of solve2.py:264-297.
"""
from __future__ import annotations

import contextlib
import importlib.util
import io
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("PW_REFERENCE_DIR", os.path.join(os.path.dirname(ROOT), "reference"))
PIPELINE = os.path.join(REF, "src", "GP", "pipeline")
RESERVED = 2
SCHEMES = ("ge", "nt", "nn")


def _load(name):
    spec = importlib.util.spec_from_file_location("ref_" + name, os.path.join(PIPELINE, name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def partition_cases(partt):
    cases = [(12, 4, 1), (40, 400, 7), (57, 64, 100), (2 + 100, 37, 1), (2 + 64, 1000, 3), (3, 8, 1)]
    out = []
    for nkey_total, quota, gran in cases:
        nkey = nkey_total - RESERVED
        tri = np.tril_indices(nkey)
        shape = tri[0].shape
        total = partt.guess_chunk_number(shape, quota, gran)
        tasks = sorted({0, total // 2, total - 1})
        for t in tasks:
            with contextlib.redirect_stdout(io.StringIO()):      # chunk_it prints its progress
                chunk = np.array(partt.get_task_chunk(shape, total, t)).reshape(-1)
            out.append((nkey_total, quota, gran, total, t, tri[0][chunk] + RESERVED, tri[1][chunk] + RESERVED))
    return out


def root_cases(djs_mod, rng):
    out = []
    for case in range(6):
        nkey = int(rng.integers(6, 60)) + RESERVED
        per = np.sort(rng.integers(0, nkey - RESERVED + 1, size=2))
        bases = np.array([RESERVED, RESERVED + per[0], RESERVED + per[1], nkey], dtype=np.int64)
        nedge = int(rng.integers(0, 3 * nkey))
        ef = rng.integers(0, nkey, size=nedge)
        et = rng.integers(0, nkey, size=nedge)
        dis = rng.random(nkey) < (0.15 * case)
        ranges = {s: (int(bases[i]), int(bases[i + 1])) for i, s in enumerate(SCHEMES)}
        ranges["cmb"] = (RESERVED, nkey)
        picked = {}
        for scheme, (lo, hi) in ranges.items():
            djs = djs_mod.DisjointSet([i for i in range(lo, hi)])
            for r, c in zip(ef, et):
                if r >= hi or r < lo or c >= hi or c < lo:
                    continue
                djs.union(r, c)
            screened = []
            for k in djs.get_cluster().values():
                for member in k:
                    if not dis[member]:
                        screened.append(member)
                        break
            picked[scheme] = np.array(list(range(RESERVED)) + screened, dtype=np.int64)
        out.append((nkey, bases, ef.astype(np.int64), et.astype(np.int64), dis, picked))
    return out


def main():
    partt = _load("partt")
    djs_mod = _load("disjoint_set")
    rng = np.random.default_rng(2024)
    arrays = {}
    pc = partition_cases(partt)
    arrays["part_meta"] = np.array([c[:5] for c in pc], dtype=np.int64)
    for i, c in enumerate(pc):
        arrays["part_from_%d" % i] = c[5].astype(np.int64)
        arrays["part_to_%d" % i] = c[6].astype(np.int64)
    rc = root_cases(djs_mod, rng)
    arrays["root_count"] = np.array(len(rc))
    for i, (nkey, bases, ef, et, dis, picked) in enumerate(rc):
        arrays["root_%d_nkey" % i] = np.array(nkey)
        arrays["root_%d_bases" % i] = bases
        arrays["root_%d_from" % i] = ef
        arrays["root_%d_to" % i] = et
        arrays["root_%d_dis" % i] = dis
        for s, idx in picked.items():
            arrays["root_%d_%s" % (i, s)] = idx
    np.savez_compressed(os.path.join(HERE, "screening_golden.npz"), **arrays)
    print("wrote screening_golden.npz: %d partition cases, %d root cases" % (len(pc), len(rc)))


if __name__ == "__main__":
    main()

"""The planner stages whose work is collision queries, on the engine, with the
pipeline's on-disk formats (src/GP/pipeline/solve2.py).

* Key-configuration screening (solve2.py:164-232).
  - Every pair (i, j) with j <= i of the predicted keys (after the two
    reserved init / goal rows) is tested with isValidTransition at the
    world's recommended resolution.  The visible pairs are the screening
    graph's edges.
  - The reference splits the lower triangle into HTCondor tasks
    (partt.py:10-35) and loops over the pairs of a task.  Here the keys stay
    on the device, and each task's pairs are decoded from their flat
    indices on the device and checked as segment batches.
  - ``edge_batch-<i>.npz`` (EDGE_FROM, EDGE_TO) is written per reference
    task, so the reference's next stage reads the files unchanged.
* Root assembly (solve2.py:234-306): the connected components of the
  screening graph within each scheme's key range.  A component's first key
  (in index order) that is not disentangled becomes a root.  All
  disentangled tests run as one batch.
* Blooming assembly (solve2.py:389-450): Q, QF, QB (QE, QEB) of the
  blooming forest.  QF marks the disentangled samples with
  PDS_FLAG_TERMINATE; all of them are tested as one batch.

The file layout follows the reference: key files hold KEYQ_OMPL (and
BASES_WITH_END), edge files EDGE_FROM / EDGE_TO (int64), PDS files Q, QF
(uint32 [n, 1]), QB and optionally QE, QEB, BLOOM_NO_TO_INDEX and
INDEX_TO_BLOOM_NO.
"""
from __future__ import annotations

import os
import pathlib

import numpy as np
import torch

from . import _lib

RESERVED = 2                          # util.RDT_FOREST_INIT_AND_GOAL_RESERVATIONS (util.py:73)
RAW_KEY_PRED_SCHEMES = ("ge", "nt", "nn")   # file_locations.py:14
PDS_FLAG_TERMINATE = 1                # forest_dijkstra.py:75


# ---------------------------------------------------------------- task partition

def guess_chunk_number(ntask: int, max_chunk_number: int, minimal_chunk_size: int) -> int:
    """partt.guess_chunk_number (partt.py:23-27)."""
    return max(1, min(int(max_chunk_number), int(ntask / float(minimal_chunk_size))))


def chunk_bounds(ntask: int, num: int) -> np.ndarray:
    """[start, end) of each task of partt.chunk_it (partt.py:10-21) over ntask
    items: chunks of float width ntask / num cut at int(k * width) by a running
    float sum, the remainder joining the last chunk.  Raises where the
    reference's own assertion fails."""
    avg = ntask / float(num)
    starts = []
    last = 0.0
    while last < ntask and len(starts) < num:
        starts.append(last)
        last += avg
    if not starts:
        raise ValueError("no tasks to partition")
    if len(starts) != num:
        raise ValueError("len(out) (%d) != %d" % (len(starts), num))
    # slices clamp at the end; the last chunk takes everything from its start on
    out = [[min(int(s), ntask), min(int(s + avg), ntask)] for s in starts]
    out[-1][1] = ntask
    return np.asarray(out, dtype=np.int64)


def tril_pairs(k):
    """(row, col) of flat index k in np.tril_indices order (row-major over j <= i)."""
    k = np.asarray(k, dtype=np.int64)
    i = np.floor((np.sqrt(8.0 * k.astype(np.float64) + 1.0) - 1.0) / 2.0).astype(np.int64)
    i = np.where(i * (i + 1) // 2 > k, i - 1, i)
    i = np.where((i + 1) * (i + 2) // 2 <= k, i + 1, i)
    return i, k - i * (i + 1) // 2


def _tril_pairs_dev(k: torch.Tensor):
    i = torch.floor((torch.sqrt(8.0 * k.to(torch.float64) + 1.0) - 1.0) / 2.0).to(torch.int64)
    i = torch.where(i * (i + 1) // 2 > k, i - 1, i)
    i = torch.where((i + 1) * (i + 2) // 2 <= k, i + 1, i)
    return i, k - i * (i + 1) // 2


def partition_screening(nkey_total: int, max_chunk_number: int, minimal_chunk_size: int, index: int | None = None):
    """solve2._partition_screening (solve2.py:78-94) for a key file of
    nkey_total rows: the number of tasks, or task `index`'s (from, to) key
    indices (int64, reserved rows offset in)."""
    nkey = nkey_total - RESERVED
    ntask = nkey * (nkey + 1) // 2
    total = guess_chunk_number(ntask, max_chunk_number, minimal_chunk_size)
    if index is None:
        return total
    s, e = chunk_bounds(ntask, total)[index]
    r, c = tril_pairs(np.arange(s, e, dtype=np.int64))
    return r + RESERVED, c + RESERVED


# ---------------------------------------------------------------- screening

def _unit_keys(uw, keys) -> torch.Tensor:
    """The keys as the screening stage converts them: calculate_visibility_pair
    with qs_are_unit_states = False applies translateToUnitState."""
    k = np.ascontiguousarray(np.asarray(keys, dtype=np.float64))
    if k.ndim != 2 or k.shape[1] != 7:
        raise ValueError("keys must be [n, 7]")
    return torch.from_numpy(uw.translate_to_unit_state(k)).to(uw._device)


def _visible(uw, U: torch.Tensor, fi: torch.Tensor, ti: torch.Tensor, vm: float) -> torch.Tensor:
    steps = uw.first_contact_steps(U.index_select(0, fi), U.index_select(0, ti), vm, _lib.PW_SEG_TRANSITION)
    return steps == _lib.PW_STEP_FREE


def screen_pairs(uw, keys, from_indices, to_indices, verify_magnitude: float | None = None,
                 batch: int = 1 << 22):
    """One screening task (solve2.py:176-183): the (EDGE_FROM, EDGE_TO) pairs of
    the given ones that isValidTransition finds visible, in input order."""
    vm = uw.recommended_cres if verify_magnitude is None else float(verify_magnitude)
    fi = np.asarray(from_indices, dtype=np.int64).reshape(-1)
    ti = np.asarray(to_indices, dtype=np.int64).reshape(-1)
    if fi.shape != ti.shape:
        raise ValueError("from and to indices differ in length")
    U = _unit_keys(uw, keys)
    keep = []
    for s in range(0, fi.shape[0], batch):
        a = torch.from_numpy(fi[s:s + batch]).to(uw._device)
        b = torch.from_numpy(ti[s:s + batch]).to(uw._device)
        keep.append(_visible(uw, U, a, b, vm).cpu().numpy())
    m = np.concatenate(keep) if keep else np.zeros(0, dtype=bool)
    return fi[m], ti[m]


def screen_keyconf(uw, keys, max_chunk_number: int = 1, minimal_chunk_size: int = 1, out_dir: str | None = None,
                   verify_magnitude: float | None = None, batch: int = 1 << 22, resume: bool = False,
                   driver=None):
    """The whole screening stage: every task of partition_screening checked on
    the device (pairs decoded from flat indices there, nothing per pair on the
    host).  Returns (EDGE_FROM, EDGE_TO) over all tasks in task order; with
    out_dir, also writes edge_batch-<task>.npz per task as the reference's
    workers do (solve2.py:226).  With resume, a task whose file already exists
    is read back instead of checked again, as the reference's rerun mode
    recomputes only the missing task outputs (solve2.py:168-187).

    The pairs are checked as the reference's rerun mode does
    (calculate_visibility_pair at verify_magnitude, solve2.py:180-183), or,
    with an ompl_compat.OmplDriver set up for the puzzle, as its workers do:
    driver.validate_motion_pairs on the OMPL-frame keys (solve2.py:218-219),
    OMPL's discrete motion rule at the driver's bounds and resolution."""
    vm = uw.recommended_cres if verify_magnitude is None else float(verify_magnitude)
    keys = np.asarray(keys, dtype=np.float64)
    nkey = keys.shape[0] - RESERVED
    if nkey <= 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    ntask = nkey * (nkey + 1) // 2
    total = guess_chunk_number(ntask, max_chunk_number, minimal_chunk_size)
    bounds = chunk_bounds(ntask, total)
    dev = uw._device
    if driver is None:
        U = _unit_keys(uw, keys)

        def visible(r, c):
            return _visible(uw, U, r, c, vm)
    else:
        P = torch.from_numpy(np.ascontiguousarray(keys)).to(dev)

        def visible(r, c):
            return driver.check_pairs(P, r, c)
    all_f, all_t = [], []
    for task, (s, e) in enumerate(bounds):
        fn = os.path.join(out_dir, "edge_batch-{}.npz".format(task)) if out_dir is not None else None
        if resume and fn is not None and os.path.isfile(fn):
            d = np.load(fn)
            all_f.append(np.asarray(d["EDGE_FROM"], dtype=np.int64))
            all_t.append(np.asarray(d["EDGE_TO"], dtype=np.int64))
            continue
        ef, et = [], []
        for s0 in range(int(s), int(e), batch):
            k = torch.arange(s0, min(int(e), s0 + batch), dtype=torch.int64, device=dev)
            r, c = _tril_pairs_dev(k)
            r, c = r + RESERVED, c + RESERVED
            vis = visible(r, c)
            ef.append(r[vis].cpu().numpy())
            et.append(c[vis].cpu().numpy())
        f = np.concatenate(ef) if ef else np.zeros(0, np.int64)
        t = np.concatenate(et) if et else np.zeros(0, np.int64)
        if fn is not None:
            os.makedirs(out_dir, exist_ok=True)
            np.savez_compressed(fn, EDGE_FROM=f, EDGE_TO=t)
        all_f.append(f)
        all_t.append(t)
    return np.concatenate(all_f), np.concatenate(all_t)


def load_edges(screen_dir: str):
    """EDGE_FROM, EDGE_TO of every edge_batch-*.npz in a directory, concatenated
    in the directory's glob order (as solve2.py:252-262)."""
    ef, et = [], []
    for fn in pathlib.Path(screen_dir).glob("edge_batch-*.npz"):
        d = np.load(fn)
        ef.append(d["EDGE_FROM"])
        et.append(d["EDGE_TO"])
    if not ef:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    return np.concatenate(ef), np.concatenate(et)


# ---------------------------------------------------------------- roots

def select_roots(lo: int, hi: int, edges_from, edges_to, disentangled) -> list[int]:
    """The roots of one key range (solve2.py:268-297): components of the edges
    with both ends in [lo, hi), ordered by their smallest key (the order in
    which DisjointSet.get_cluster meets them), each giving its first key in
    index order that is not disentangled (none if all are)."""
    n = int(hi) - int(lo)
    if n <= 0:
        return []
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    ef = np.asarray(edges_from, dtype=np.int64).reshape(-1)
    et = np.asarray(edges_to, dtype=np.int64).reshape(-1)
    m = (ef >= lo) & (ef < hi) & (et >= lo) & (et < hi)
    g = coo_matrix((np.ones(int(m.sum()), np.int8), (ef[m] - lo, et[m] - lo)), shape=(n, n))
    ncomp, lab = connected_components(g, directed=False)
    members = np.arange(n)
    first_member = np.full(ncomp, n, dtype=np.int64)
    np.minimum.at(first_member, lab, members)
    cand = members[~np.asarray(disentangled, dtype=bool)[lo:hi]]
    first_free = np.full(ncomp, n, dtype=np.int64)
    np.minimum.at(first_free, lab[cand], cand)
    order = np.argsort(first_member, kind="stable")
    return [int(first_free[c]) + int(lo) for c in order if first_free[c] < n]


def key_disentangled(uw, keys) -> np.ndarray:
    """isDisentangled of every key after translateOMPLStateToUnitState (one batch)."""
    k = np.ascontiguousarray(np.asarray(keys, dtype=np.float64))
    if k.shape[0] == 0:
        return np.zeros(0, dtype=bool)
    u = torch.from_numpy(uw.translate_ompl_to_unit(k)).to(uw._device)
    return uw.is_disentangled_states(u).cpu().numpy().astype(bool)


def assemble_roots(uw, keys, bases, edges_from, edges_to, schemes=RAW_KEY_PRED_SCHEMES, disentangled=None) -> dict:
    """solve2.assemble_roots for one puzzle: {scheme: screened KEYQ_OMPL}, the
    reserved rows first, for every scheme's range and for 'cmb' (all keys)."""
    keys = np.asarray(keys, dtype=np.float64)
    nkey = keys.shape[0]
    dis = key_disentangled(uw, keys) if disentangled is None else np.asarray(disentangled, dtype=bool)
    ranges = {s: (int(bases[i]), int(bases[i + 1])) for i, s in enumerate(schemes)}
    ranges["cmb"] = (RESERVED, nkey)
    out = {}
    for scheme, (lo, hi) in ranges.items():
        idx = list(range(RESERVED)) + select_roots(lo, hi, edges_from, edges_to, dis)
        out[scheme] = keys[idx]
    return out


# ---------------------------------------------------------------- blooming forest

def pds_flags(uw, Q) -> np.ndarray:
    """QF of solve2.py:432-435: uint32 [n, 1], PDS_FLAG_TERMINATE where the
    sample is disentangled in the unit frame (OMPL conversion)."""
    dis = key_disentangled(uw, Q)
    return (dis.astype(np.uint32) * np.uint32(PDS_FLAG_TERMINATE)).reshape(-1, 1)


def assemble_blooming(uw, bloom_dir: str, pds_fn: str) -> dict:
    """solve2.assemble_blooming for one puzzle: reads bloom-from_<i>.npz (BLOOM
    [m, 7] and optional BLOOM_EDGE [2, m - 1]) in sorted file-name order,
    writes the PDS file and returns its arrays."""
    fn_list = sorted(pathlib.Path(bloom_dir).glob("bloom-from_*.npz"))
    bloom_no_to_index = np.full((len(fn_list)), -1, dtype=np.int32)
    index_to_bloom_no, q_list, qe_list, qb, qeb = [], [], [], [], []
    tree_base = edge_base = 0
    for fn in fn_list:
        d = np.load(fn)
        bloom = d["BLOOM"]
        if bloom.shape[0] == 0:
            continue
        if bloom.shape[1] != 7:
            raise ValueError("%s's shape is %s" % (fn, bloom.shape))
        name = fn.name
        bloom_id = int(name[len("bloom-from_"):-len(".npz")])
        bloom_no_to_index[bloom_id] = len(index_to_bloom_no)
        index_to_bloom_no.append(bloom_id)
        q_list.append(bloom)
        if "BLOOM_EDGE" in d and qe_list is not None:
            edges = np.transpose(d["BLOOM_EDGE"]) + tree_base
            qe_list.append(edges)
            qeb.append(edge_base)
            edge_base += int(edges.shape[0])
        else:
            qe_list = None
        qb.append(tree_base)
        tree_base += int(bloom.shape[0])
    Q = np.concatenate(q_list, axis=0)
    out = {"Q": Q, "QF": pds_flags(uw, Q), "QB": qb}
    if qe_list:
        QE = np.concatenate(qe_list, axis=0)
        if QE.shape[0] != Q.shape[0] - len(qb):
            raise ValueError("broken tree edges: %d edges for %d samples in %d trees" %
                             (QE.shape[0], Q.shape[0], len(qb)))
        out.update(QE=QE, QEB=qeb)
    out.update(BLOOM_NO_TO_INDEX=bloom_no_to_index, INDEX_TO_BLOOM_NO=index_to_bloom_no)
    np.savez_compressed(pds_fn, **out)
    return out

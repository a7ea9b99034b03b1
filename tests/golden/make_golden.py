"""Regenerates the golden fixtures in tests/golden/ by running the reference's own
CPU SCAN build (scan-query, BIT_VEC variant, single thread) through
oracle/ref_harness on small seeded graphs and hand-built graphs.

Needs the reference tree (to build oracle/_ref) and libaccx.so (for the seeded
host generators); run from the repository root:

    python tests/golden/make_golden.py

Each fixture <name>.npz holds the graph (off, dst), the query (eps, mu) and the
reference's outputs: cnn (= 2 + common-neighbour count per CSR entry), sim,
label (final, 0/1/2), cluster (min-id cluster of cores, -1 otherwise) and the
bytes of its scanxp-result-<eps>-<mu>.txt file.  edge_list_converter.npz holds a
text edge list and the two files the reference's converter writes for it.

Two JSON fixtures too large to keep as arrays, or from another reference tool:
  rmat16_e02_mu5_digests.json  the plain CPU config (R-MAT scale 16, edge factor
      16, seed 1; eps 0.2, mu 5): sha256 digests (and sums) of the reference
      build's cnn, sim, label and cluster arrays and of its result file;
  vertex_ranges.json  the reference's ComputeVertexRangeAccumulatedFilteredDegree
      ranges (oracle/_ref/ref_ranges) for every golden graph and R-MAT 16, at
      several part counts.

    python tests/golden/make_golden.py [npz] [converter] [digests] [ranges]

(no argument: all of them).
"""
import hashlib
import json
import subprocess
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from acctricnt_gb300 import accx  # noqa: E402
from oracle import oracle  # noqa: E402


def csr_from_edges(n, edges):
    adj = [set() for _ in range(n)]
    for a, b in edges:
        if a != b:
            adj[a].add(b)
            adj[b].add(a)
    off = np.zeros(n + 1, np.uint32)
    dst = []
    for u in range(n):
        nb = sorted(adj[u])
        dst.extend(nb)
        off[u + 1] = off[u] + len(nb)
    return off, np.array(dst, np.int32)


def clique(vs):
    return [(a, b) for i, a in enumerate(vs) for b in vs[i + 1:]]


def hand_graphs():
    g = {}
    g["path"] = (csr_from_edges(12, [(i, i + 1) for i in range(11)]), 0.5, 2)
    g["star"] = (csr_from_edges(40, [(0, i) for i in range(1, 40)]), 0.3, 3)
    g["clique"] = (csr_from_edges(16, clique(list(range(16)))), 0.8, 5)
    # two 8-cliques joined through a vertex adjacent to two members of each: a hub
    two = clique(list(range(1, 9))) + clique(list(range(10, 18))) + [(9, 1), (9, 2), (9, 10), (9, 11)]
    g["two_cliques_hub"] = (csr_from_edges(19, two), 0.6, 4)
    # isolated first and last vertices around a dense core
    iso = clique(list(range(1, 12))) + [(3, 14), (5, 14), (14, 15)]
    g["isolated_ends"] = (csr_from_edges(20, iso), 0.5, 3)
    # one vertex of degree 600 next to low-degree vertices (skew ratio far above 50)
    rng = np.random.default_rng(7)
    sk = [(0, i) for i in range(1, 601)] + [(int(a), int(b)) for a, b in rng.integers(1, 601, size=(900, 2))]
    sk += clique(list(range(1, 13)))
    g["skew_hub"] = (csr_from_edges(601, sk), 0.3, 3)
    g["empty_edges"] = (csr_from_edges(5, []), 0.5, 2)
    return g


def seeded_graphs():
    g = {}
    g["rmat10_e02_mu5"] = (accx.generate_host(accx.rmat_params(10, 16, seed=1)), 0.2, 5)
    g["rmat11_e05_mu3"] = (accx.generate_host(accx.rmat_params(11, 16, seed=2)), 0.5, 3)
    g["rmat11_e08_mu2"] = (accx.generate_host(accx.rmat_params(11, 16, seed=2)), 0.8, 2)
    g["er2000_e015_mu2"] = (accx.generate_host(accx.er_params(2000, 24, seed=3)), 0.15, 2)
    g["chunglu4000_e025_mu4"] = (accx.generate_host(accx.chung_lu_params(4000, 12, 2.1, 800, seed=5)), 0.25, 4)
    g["rmat12_e03_mu4"] = (accx.generate_host(accx.rmat_params(12, 8, seed=4)), 0.3, 4)
    return g


def edge_list_text():
    """A text edge list with comments, self loops, reversed copies of edges
    (dropped by the converter), isolated ids below the largest one and tab
    separators; no repeated (i < j) pair and no blank line (the reference reads
    uninitialised ids for a line without two numbers)."""
    rng = np.random.default_rng(11)
    lines = ["# Directed graph (each unordered pair on one line)", "# FromNodeId\tToNodeId"]
    pairs = set()
    while len(pairs) < 400:
        a, b = (int(x) for x in rng.integers(0, 180, 2))
        if a != b:
            pairs.add((min(a, b), max(a, b)))
    for a, b in sorted(pairs, key=lambda p: (p[1] * 7 + p[0]) % 97):
        lines.append("%d\t%d" % (a, b))
        if (a + b) % 5 == 0:
            lines.append("%d %d" % (b, a))  # reversed copy
    lines += ["7 7", "199 250", "# trailing comment", "3 260"]
    return ("\n".join(lines) + "\n").encode()


def edge_list_fixture():
    """Runs the reference converter (oracle/_ref/edge-list-converter) on the text."""
    import subprocess
    d = tempfile.mkdtemp(prefix="golden_el_")
    src = os.path.join(d, "edges.txt")
    with open(src, "wb") as f:
        f.write(edge_list_text())
    exe = os.path.join(ROOT, "oracle", "_ref", "edge-list-converter")
    subprocess.run([exe, src, os.path.join(d, "b_degree.bin"), os.path.join(d, "b_adj.bin")], check=True,
                   capture_output=True)
    out = {}
    for k in ("edges.txt", "b_degree.bin", "b_adj.bin"):
        with open(os.path.join(d, k), "rb") as f:
            out[k.replace(".", "_")] = np.frombuffer(f.read(), np.uint8)
    np.savez_compressed(os.path.join(HERE, "edge_list_converter.npz"), **out)
    print("edge_list_converter      text=%d bytes degree=%d bytes adj=%d bytes" % (
        len(out["edges_txt"]), len(out["b_degree_bin"]), len(out["b_adj_bin"])))


def sha256(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def plain_config_graph():
    """R-MAT scale 16, edge factor 16, (0.57, 0.19, 0.19, 0.05), seed 1."""
    return accx.generate_host(accx.rmat_params(16, 16, seed=1))


def digests_fixture():
    off, dst = plain_config_graph()
    eps, mu = 0.2, 5
    d = tempfile.mkdtemp(prefix="golden_dg_")
    accx.write_graph_dir(d, off, dst)
    ref = oracle.run_reference(d, eps, mu, os.path.join(d, "dump"))
    fn = "scanxp-result-%s-%d.txt" % (oracle.eps_string(eps), mu)
    with open(os.path.join(d, fn), "rb") as f:
        result = f.read()
    out = {"graph": "R-MAT scale 16, edge factor 16, (0.57,0.19,0.19,0.05), seed 1", "n": int(len(off) - 1),
           "m": int(len(dst)), "eps": eps, "mu": mu, "graph_sha256": {"off": sha256(off), "dst": sha256(dst)},
           "sha256": {k: sha256(ref[k]) for k in ("cnn", "sim", "label", "cluster")},
           "sums": {k: int(ref[k].astype(np.int64).sum()) for k in ("cnn", "sim", "label", "cluster")},
           "result_name": fn, "result_sha256": hashlib.sha256(result).hexdigest(), "result_bytes": len(result)}
    with open(os.path.join(HERE, "rmat16_e02_mu5_digests.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("rmat16_e02_mu5_digests    n=%d m=%d result=%d bytes" % (out["n"], out["m"], len(result)))


RANGE_PARTS = (1, 2, 3, 4, 7, 8)


def ranges_fixture():
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_ranges")
    graphs = {name: (off, dst) for name, ((off, dst), _, _) in list(hand_graphs().items()) + list(seeded_graphs().items())}
    graphs["rmat16"] = plain_config_graph()
    out = {"parts": list(RANGE_PARTS), "ranges": {}}
    for name, (off, dst) in sorted(graphs.items()):
        d = tempfile.mkdtemp(prefix="golden_vr_")
        accx.write_graph_dir(d, off, dst)
        r = subprocess.run([exe, d] + [str(p) for p in RANGE_PARTS], check=True, capture_output=True, text=True)
        out["ranges"][name] = [[int(x) for x in line.split()] for line in r.stdout.strip().splitlines()]
    with open(os.path.join(HERE, "vertex_ranges.json"), "w") as f:
        json.dump(out, f)
    print("vertex_ranges             %d graphs x %d part counts" % (len(out["ranges"]), len(RANGE_PARTS)))


def main():
    what = set(sys.argv[1:]) or {"npz", "converter", "digests", "ranges"}
    oracle.build()
    if not oracle.have_reference():
        raise SystemExit("reference build not available; cannot regenerate fixtures")
    if "digests" in what:
        digests_fixture()
    if "ranges" in what:
        ranges_fixture()
    if "npz" in what:
        npz_fixtures()
    if "converter" in what:
        edge_list_fixture()


def npz_fixtures():
    cases = {}
    cases.update(hand_graphs())
    cases.update(seeded_graphs())
    for name, ((off, dst), eps, mu) in sorted(cases.items()):
        d = tempfile.mkdtemp(prefix="golden_")
        accx.write_graph_dir(d, off, dst)
        ref = oracle.run_reference(d, eps, mu, os.path.join(d, "dump"))
        fn = "scanxp-result-%s-%d.txt" % (oracle.eps_string(eps), mu)
        with open(os.path.join(d, fn), "rb") as f:
            result = f.read()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), off=off, dst=dst, eps=np.float64(eps),
                            mu=np.int32(mu), cnn=ref["cnn"], sim=ref["sim"], label=ref["label"],
                            cluster=ref["cluster"], result=np.frombuffer(result, np.uint8), result_name=fn)
        print("%-24s n=%-6d m=%-7d cores=%-5d hubs=%-4d pairs-lines=%d" % (
            name, len(off) - 1, len(dst), int((ref["label"] == 1).sum()), int((ref["label"] == 2).sum()),
            result.count(b"\nn ")))


if __name__ == "__main__":
    main()

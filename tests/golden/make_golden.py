"""Regenerates the golden fixtures in tests/golden/ by running the reference's own
CPU SCAN build (scan-query, BIT_VEC variant, single thread) through
oracle/ref_harness on small seeded graphs and hand-built graphs.

Needs the reference tree (to build oracle/_ref) and libaccx.so (for the seeded
host generators); run from the repository root:

    python tests/golden/make_golden.py

Each fixture <name>.npz holds the graph (off, dst), the query (eps, mu) and the
reference's outputs: cnn (= 2 + common-neighbour count per CSR entry), sim,
label (final, 0/1/2), cluster (min-id cluster of cores, -1 otherwise) and the
bytes of its scanxp-result-<eps>-<mu>.txt file.
"""
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


def main():
    oracle.build()
    if not oracle.have_reference():
        raise SystemExit("reference build not available; cannot regenerate fixtures")
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

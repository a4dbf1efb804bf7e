"""Link sets for the cellular automaton on caller inputs (CellularAutomaton::run
takes any basis/follower/pt arrays, CellularAutomaton.h:43-49).

random_links(): a directed acyclic link set over n_triplets triplets placed
on levels; links go from a lower to a higher level, skipping levels at
random, with several bases per follower and a few repeated links, unlike the
chain's own links (one layer triplet to the next).  pt values come from a
small set so that ties of |dpt| occur.
"""
import numpy as np


def random_links(seed: int, n_triplets: int = 3000, n_levels: int = 7, links_per_triplet: float = 2.0,
                 sort_by_basis: bool = True):
    rng = np.random.default_rng(seed)
    level = np.sort(rng.integers(0, n_levels, n_triplets))
    n_links = int(links_per_triplet * n_triplets)
    b = rng.integers(0, n_triplets, 4 * n_links)
    f = rng.integers(0, n_triplets, 4 * n_links)
    keep = level[b] < level[f]
    b, f = b[keep][:n_links], f[keep][:n_links]
    dup = rng.integers(0, b.size, b.size // 50)  # a few links given twice
    b, f = np.concatenate([b, b[dup]]), np.concatenate([f, f[dup]])
    if sort_by_basis:
        order = np.lexsort((f, b))
        b, f = b[order], f[order]
    pt = rng.choice(np.float32([10.0, 12.5, 20.0, 33.25, 50.0, 75.5, 100.0, 150.0]), n_triplets)
    pt = pt * (1 + (rng.random(n_triplets) < 0.5) * rng.random(n_triplets).astype(np.float32) * 1e-3)
    return b.astype(np.uint32), f.astype(np.uint32), pt.astype(np.float32)

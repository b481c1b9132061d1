"""Shared test fixtures: random trees, random SOP operators and generic states."""
import numpy as np

from ttns_lib_gb300.model import SOPOperator, Topology, _NTree, _flatten


def random_tree(rng, leaf_dims, max_children=3, chi=None):
    """Random pre-order tree over the given leaves; chi=None keeps every bond full rank."""
    big = 10 ** 6 if chi is None else chi
    nodes = [_NTree(big, phys=int(d), mode=k) for k, d in enumerate(leaf_dims)]
    rng.shuffle(nodes)
    while len(nodes) > 1:
        k = int(rng.integers(2, min(max_children, len(nodes)) + 1))
        grp, nodes = nodes[:k], nodes[k:]
        parent = _NTree(big)
        parent.kids = grp
        pos = int(rng.integers(0, len(nodes) + 1))
        nodes.insert(pos, parent)
    root = _NTree(1)
    if nodes[0].phys is not None:
        root.kids = [nodes[0]]
    else:
        root.kids = nodes[0].kids
    topo = _flatten(root)
    if chi is None:
        topo = full_rank(topo)
    return topo


def full_rank(topo):
    """Set every bond to min(dim below, dim above) so the tree spans the whole space."""
    n = topo.nnodes
    below = [1] * n
    for i in range(n - 1, -1, -1):
        if topo.is_leaf(i):
            below[i] = int(topo.leaf_dim[i])
        else:
            p = 1
            for c in topo.children[i]:
                p *= below[c]
            below[i] = p
    total = below[0]
    hr = np.array([1] + [min(below[i], total // below[i]) for i in range(1, n)], dtype=np.int32)
    return Topology(topo.parent, hr, topo.leaf_mode, topo.leaf_dim)


def rand_herm(rng, d):
    a = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    return (a + a.conj().T) / 2


def random_sop(rng, mode_dims, nterms=12, max_modes=3, share_prob=0.4, dup=True):
    """Random Hermitian SOP with shared operators, identity-only terms and duplicates."""
    nm = len(mode_dims)
    H = SOPOperator(nterms, mode_dims)
    supports = []
    for r in range(nterms):
        if r == nterms - 1 and dup and nterms > 2:
            supports.append(list(supports[0]))
            continue
        k = int(rng.integers(0, max_modes + 1))
        supports.append(sorted(rng.choice(nm, size=min(k, nm), replace=False).tolist()))
    for m in range(nm):
        users = [r for r in range(nterms) if m in supports[r]]
        rng.shuffle(users)
        while users:
            take = 1
            if len(users) > 1 and rng.random() < share_prob:
                take = int(rng.integers(2, len(users) + 1))
            grp, users = users[:take], users[take:]
            H.bind_dense(rand_herm(rng, mode_dims[m]), grp, m)
    H.coeffs = rng.uniform(-1.0, 1.0, size=nterms).astype(np.complex128)
    return H


def generic_state(topo, rng):
    """Random isometries below a random normalised root: every bond well populated."""
    st = []
    for i in range(topo.nnodes):
        d, r = topo.node_shape(i)
        a = rng.normal(size=(d, r)) + 1j * rng.normal(size=(d, r))
        if i != 0:
            a, _ = np.linalg.qr(a)
        else:
            a /= np.linalg.norm(a)
        st.append(np.ascontiguousarray(a))
    return st


def random_case(seed, chi=None, max_children=None):
    """A random tree, a random SOP operator of random shape (number of terms, modes per
    term, sharing, duplicates) and a generic state.  The shapes include groups that mix
    terms acting below a node with terms that are the identity there."""
    rng = np.random.default_rng(seed)
    dims = [int(x) for x in rng.integers(2, 4, size=int(rng.integers(3, 6)))]
    mc = int(rng.integers(2, 4)) if max_children is None else max_children
    topo = random_tree(rng, dims, max_children=mc, chi=chi)
    H = random_sop(rng, dims, nterms=int(rng.integers(3, 12)))
    st = generic_state(topo, rng)
    return topo, H, st, dims

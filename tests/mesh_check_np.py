"""numpy restatement of the mesh check (test helper): components of the face graph across shared
edges, orientation defects (an edge whose two faces run it in the same direction), boundary edges,
halfedges on edges with three or more faces, degenerate faces and boundary vertices."""
import numpy as np


def mesh_check_np(nv, faces, P):
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    f = np.asarray(faces, np.int64).reshape(-1, P)
    nf = len(f)
    if nf == 0:
        return dict(components=0, orientation_defects=0, boundary_edges=0, nonmanifold_halfedges=0,
                    degenerate_faces=0, boundary_vertices=0)
    a = f.reshape(-1)
    b = np.roll(f, -1, axis=1).reshape(-1)
    face_of = np.repeat(np.arange(nf), P)
    key = (np.minimum(a, b) << 32) | np.maximum(a, b)
    order = np.argsort(key, kind="stable")
    _, start, counts = np.unique(key[order], return_index=True, return_counts=True)
    two = counts == 2
    i0, i1 = order[start[two]], order[start[two] + 1]
    g = coo_matrix((np.ones(len(i0)), (face_of[i0], face_of[i1])), shape=(nf, nf))
    ncomp, _ = connected_components(g, directed=False)
    one = order[start[counts == 1]]
    bverts = np.unique(np.concatenate([a[one], b[one]])) if len(one) else np.zeros(0)
    deg = np.zeros(nf, bool)
    for x in range(P):
        for y in range(x + 1, P):
            deg |= f[:, x] == f[:, y]
    return dict(components=int(ncomp), orientation_defects=int((a[i0] == a[i1]).sum()),
                boundary_edges=int((counts == 1).sum()), nonmanifold_halfedges=int(counts[counts >= 3].sum()),
                degenerate_faces=int(deg.sum()), boundary_vertices=int(len(bverts)))

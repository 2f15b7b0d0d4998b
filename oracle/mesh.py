"""Structured simplex grid, compartments and interfaces (oracle side, test infrastructure).

Restates dune/copasi/grid/make_multi_domain_grid.hh:
  * :76-91  ``grid.cells`` (default 1 per axis), ``grid.origin`` (default 0),
    ``grid.extensions`` (default 1) -> StructuredGridFactory::createSimplexGrid, i.e. the
    Kuhn split of every cube: one simplex per permutation p of the axes, walking
    corner 0 -> +e_p0 -> +e_p1 ... (2 triangles per square, 6 tetrahedra per cube);
  * :96-100 ``grid.refinement_level`` global refinements.  Red refinement of the Kuhn
    split reproduces the Kuhn split of the grid with twice the cells per axis, so
    level r is built directly as cells * 2**r;
  * :118-154,166-194 compartment marking: each compartment's expression is evaluated
    at the cell centre and the cell belongs to the compartment when the value != 0;
    compartment ids follow the order of ``[compartments]`` in the configuration;
  * :66-76 ``grid.path``: a Gmsh file (read_gmsh), whose physical entities become the cell
    data ``gmsh_id`` visible to the compartment expressions (:112-132).
"""

import itertools

import numpy as np

from . import expr as E

AXES = ("x", "y", "z")


def structured_simplex(dim, cells, origin, extensions):
    cells = [int(c) for c in cells]
    origin = np.asarray(origin, float)
    ext = np.asarray(extensions, float)
    npts = [c + 1 for c in cells]
    # lexicographic vertex numbering, x fastest
    axes = [np.linspace(origin[d], origin[d] + ext[d], npts[d]) for d in range(dim)]
    grids = np.meshgrid(*axes, indexing="ij")
    coords = np.stack([g.transpose(tuple(reversed(range(dim)))).ravel() for g in grids], axis=1)
    strides = [1]
    for d in range(1, dim):
        strides.append(strides[-1] * npts[d - 1])
    strides = np.asarray(strides, np.int64)
    idx = np.stack(np.meshgrid(*[np.arange(c) for c in cells], indexing="ij"), axis=-1)
    idx = idx.transpose(tuple(reversed(range(dim))) + (dim,)).reshape(-1, dim)
    base = idx @ strides
    simplices = []
    perms = list(itertools.permutations(range(dim)))
    # cube-major ordering: for each cube, one simplex per permutation
    per_cube = []
    for p in perms:
        verts = [np.zeros(dim, np.int64)]
        cur = np.zeros(dim, np.int64)
        for ax in p:
            cur = cur.copy()
            cur[ax] = 1
            verts.append(cur)
        offs = np.array([v @ strides for v in verts], np.int64)
        per_cube.append(base[:, None] + offs[None, :])
    simplices = np.stack(per_cube, axis=1).reshape(-1, dim + 1)
    return coords, simplices


def read_gmsh(path, dim):
    """Gmsh MSH 2.x ASCII file (the format Dune's GmshReader reads,
    make_multi_domain_grid.hh:66-76): nodes in file order (ids mapped to 0..n-1); the
    elements of the grid's dimension (type 2 triangles in 2D, type 4 tetrahedra in 3D) in
    file order; lower-dimensional elements are skipped; the first tag of an element is its
    physical entity, exposed as the cell data ``gmsh_id``.  Returns (coords, cells, gmsh_id).
    """
    with open(path) as f:
        lines = [ln.strip() for ln in f]
    i = 0
    coords = None
    cells, phys = [], []
    idmap = {}
    want = 2 if dim == 2 else 4
    while i < len(lines):
        tag = lines[i]
        if tag == "$MeshFormat":
            ver = lines[i + 1].split()
            if not ver[0].startswith("2") or ver[1] != "0":
                raise ValueError("only ASCII Gmsh MSH 2.x files are supported")
            i += 3
        elif tag == "$Nodes":
            n = int(lines[i + 1])
            coords = np.zeros((n, dim))
            for k in range(n):
                parts = lines[i + 2 + k].split()
                idmap[int(parts[0])] = k
                coords[k] = [float(v) for v in parts[1:1 + dim]]
            i += n + 3
        elif tag == "$Elements":
            n = int(lines[i + 1])
            for k in range(n):
                parts = [int(v) for v in lines[i + 2 + k].split()]
                typ, ntags = parts[1], parts[2]
                if typ != want:
                    continue
                phys.append(parts[3] if ntags > 0 else 0)
                cells.append([idmap[v] for v in parts[3 + ntags:3 + ntags + dim + 1]])
            i += n + 3
        else:
            i += 1
    if coords is None or not cells:
        raise ValueError("Gmsh file without nodes or %dD elements: %r" % (dim, path))
    return coords, np.asarray(cells, np.int64), np.asarray(phys, float)


class Mesh:
    def __init__(self, coords, cells, cell_data=None):
        self.coords = np.ascontiguousarray(coords, float)
        self.cells = np.ascontiguousarray(cells, np.int64)
        self.dim = self.coords.shape[1]
        self.nv = self.coords.shape[0]
        self.ne = self.cells.shape[0]
        self.cell_data = cell_data or {}

    @classmethod
    def from_config(cls, cfg):
        """cfg: the ``grid`` ParameterTree."""
        if cfg.has_key("path"):
            dim = cfg.get_int("dimension", 2)
            if cfg.get_int("refinement_level", 0) != 0:
                raise NotImplementedError("refinement of Gmsh grids is not supported")
            coords, cells, phys = read_gmsh(cfg.get("path"), dim)
            return cls(coords, cells, {"gmsh_id": phys})
        if cfg.has_key("dimension"):
            dim = cfg.get_int("dimension")
        elif cfg.has_key("extensions"):
            dim = len(cfg.get_floats("extensions"))
        else:
            dim = 2
        if dim not in (2, 3):
            raise NotImplementedError("only 2D triangles and 3D tetrahedra")
        cells = [int(c) for c in cfg.get_floats("cells", [1] * dim)]
        ext = cfg.get_floats("extensions", [1.0] * dim)
        org = cfg.get_floats("origin", [0.0] * dim)
        level = cfg.get_int("refinement_level", 0)
        cells = [c * (2 ** level) for c in cells]
        return cls(*structured_simplex(dim, cells, org, ext))

    def centers(self):
        return self.coords[self.cells].mean(axis=1)

    def volumes(self):
        v0 = self.coords[self.cells[:, 0]]
        B = np.stack([self.coords[self.cells[:, k]] - v0 for k in range(1, self.dim + 1)], axis=2)
        det = np.linalg.det(B)
        fact = 1.0 if self.dim == 2 else 1.0
        return np.abs(det) / (2.0 if self.dim == 2 else 6.0) * fact

    def faces(self):
        """All codim-1 faces: (face_vertices sorted [nf, dim], elem0, localface0, elem1 or -1, localface1)."""
        d = self.dim
        ne = self.ne
        loc = []
        for k in range(d + 1):
            loc.append([j for j in range(d + 1) if j != k])  # face opposite local vertex k
        fv = np.concatenate([self.cells[:, lf] for lf in loc], axis=0)
        owner = np.tile(np.arange(ne), d + 1)
        lface = np.repeat(np.arange(d + 1), ne)
        key = np.sort(fv, axis=1)
        order = np.lexsort(tuple(key[:, j] for j in reversed(range(d))))
        key = key[order]
        owner = owner[order]
        lface = lface[order]
        n = key.shape[0]
        # a face shared by two cells appears twice consecutively after the sort
        start = np.ones(n, bool)
        start[1:] = np.any(key[1:] != key[:-1], axis=1)
        first = np.nonzero(start)[0]
        nxt = first + 1
        paired = np.zeros(first.shape[0], bool)
        ok = nxt < n
        paired[ok] = ~start[nxt[ok]]
        e0 = owner[first].copy()
        l0 = lface[first].copy()
        e1 = np.full(first.shape[0], -1, np.int64)
        l1 = np.full(first.shape[0], -1, np.int64)
        e1[paired] = owner[nxt[paired]]
        l1[paired] = lface[nxt[paired]]
        swap = paired & (e1 < e0)
        e0[swap], e1[swap] = e1[swap], e0[swap].copy()
        l0[swap], l1[swap] = l1[swap], l0[swap].copy()
        return key[first], e0, l0, e1, l1


def mark_compartments(mesh, comp_cfg, context):
    """Return (names, mask[ncomp, ne]) evaluating each expression at the cell centres."""
    names = comp_cfg.sub_keys()
    ctr = mesh.centers()
    env = dict(mesh.cell_data)       # cell data keys are variables (make_multi_domain_grid.hh:124-132)
    for d in range(3):
        env["position_" + AXES[d]] = ctr[:, d] if d < mesh.dim else 0.0
    masks = []
    for name in names:
        sub = comp_cfg.sub(name)
        typ = sub.get("type", "expression")
        if typ != "expression":
            raise NotImplementedError("compartment type %r" % typ)
        ex = E.Expression(sub["expression"], context)
        val = np.broadcast_to(np.asarray(ex(env), float), (mesh.ne,))
        masks.append(val != 0.0)
    return names, np.asarray(masks, bool).reshape(len(names), mesh.ne)

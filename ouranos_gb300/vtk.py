"""VTK output of the flux moments, the file the reference's output_results
writes through deal.II DataOut (src/ouranos.cc:211-253): one legacy-format
.vtk file with every cell as its own quad / hexahedron (DG fields are
discontinuous, so vertices are not shared), the moments at the cell corners as
point data and the cell averages as cell data.  Headless: no graphics API.
"""
import numpy as np


def write_vtk(path, problem, flux, names=None, group=0):
    """Write `flux` ([mom][dof] for one group, lexicographic cells) to `path`."""
    dim, p = problem.dim, problem.fe_order
    p1 = p + 1
    n = p1 ** dim
    nc = problem.total_cells
    nm = problem.quad.n_mom
    flux = np.asarray(flux, dtype=np.float64).reshape(nm, nc, n)
    nx = list(problem.n_cells) + [1] * (3 - dim)
    lo = np.array(list(problem.lower) + [0.0] * (3 - dim))
    hi = np.array(list(problem.upper) + [0.0] * (3 - dim))
    h = (hi - lo) / np.array(nx)
    idx = np.arange(nc)
    ijk = np.stack([idx % nx[0], (idx // nx[0]) % nx[1], idx // (nx[0] * nx[1])], axis=1)
    # corner k (VTK order) -> local corner bits (x, y, z) and local dof index
    if dim == 2:
        corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)]
        ctype = 9  # VTK_QUAD
    else:
        corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
                   (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
        ctype = 12  # VTK_HEXAHEDRON
    nv = len(corners)
    pts = np.zeros((nc, nv, 3))
    dof_of_corner = []
    for k, (a, b, c) in enumerate(corners):
        pts[:, k, :] = lo + (ijk + np.array([a, b, c])) * h
        dof_of_corner.append(a * p + p1 * (b * p) + (p1 * p1 * (c * p) if dim == 3 else 0))
    names = names or ["phi_%d_g%d" % (m, group) for m in range(nm)]
    with open(path, "w") as f:
        f.write("# vtk DataFile Version 3.0\nouranos_gb300 flux moments\nASCII\n")
        f.write("DATASET UNSTRUCTURED_GRID\nPOINTS %d double\n" % (nc * nv))
        np.savetxt(f, pts.reshape(-1, 3), fmt="%.9g")
        f.write("CELLS %d %d\n" % (nc, nc * (nv + 1)))
        conn = np.hstack([np.full((nc, 1), nv), np.arange(nc * nv).reshape(nc, nv)])
        np.savetxt(f, conn, fmt="%d")
        f.write("CELL_TYPES %d\n" % nc)
        np.savetxt(f, np.full(nc, ctype), fmt="%d")
        f.write("POINT_DATA %d\n" % (nc * nv))
        for m in range(nm):
            f.write("SCALARS %s double 1\nLOOKUP_TABLE default\n" % names[m])
            np.savetxt(f, flux[m][:, dof_of_corner].reshape(-1), fmt="%.12g")
        f.write("CELL_DATA %d\n" % nc)
        for m in range(nm):
            f.write("SCALARS %s_mean double 1\nLOOKUP_TABLE default\n" % names[m])
            np.savetxt(f, flux[m].mean(axis=1), fmt="%.12g")
    return path


def read_vtk_point_data(path):
    """Minimal reader of the files write_vtk produces (for tests)."""
    out = {}
    with open(path) as f:
        lines = f.read().split("\n")
    i = 0
    while i < len(lines):
        ln = lines[i]
        if ln.startswith("POINT_DATA"):
            npts = int(ln.split()[1])
            i += 1
            while i < len(lines) and lines[i].startswith("SCALARS"):
                name = lines[i].split()[1]
                vals = np.array([float(v) for v in lines[i + 2:i + 2 + npts]])
                out[name] = vals
                i += 2 + npts
            continue
        i += 1
    return out

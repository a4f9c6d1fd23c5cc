"""Generate the golden fixtures under tests/golden/ from the reference's own
test sources and quadrature tables, read as plain text.

The reference (Rombur/ouranos) cannot be built here (deal.II, Trilinos, p4est,
boost and MPI are absent), so its numbers reach the test-suite this way:

* ``ls_tables.json``     -- level-symmetric direction cosines and per-point
                             weights, ``src/LS.cc:14-665``.
* ``glc_gauss.json``     -- Gauss-Legendre nodes/weights used by the GLC
                             quadrature, ``src/GLC.cc:60-1285`` (30 digits).
* ``rt_golden.json``     -- the 64-value scalar-flux golden vector and the
                             problem it solves, ``tests/RadiativeTransfer_test.cc:84-152``
                             with ``tests/rt_*.inp``.
* ``quadrature_facts.json`` -- most-normal sets, moment orders and first
                             directions, ``tests/RTQuadrature_test.cc:21-165``.
* ``fecell_facts.json``  -- every FE matrix entry and normal the FECell test
                             pins, ``tests/FECell_test.cc:23-297``.
* ``inputs.json``        -- the reference's ``.inp`` fixtures verbatim plus the
                             values its Geometry/material tests expect
                             (``tests/Geometry_test.cc``, ``tests/RTMaterialProperties_test.cc``).

Run:  python tests/golden/make_golden.py <reference_root>
(or with the root in the environment variable OURANOS_REFERENCE_ROOT).  The
output is committed; the test-suite never reads the reference tree at run
time.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _read(root, rel):
    with open(os.path.join(root, rel)) as f:
        return f.read()


def _strip_comments(src):
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def _num(tok):
    # long decimal literals: keep 30 significant characters, python float rounds
    tok = tok.strip()
    return float(tok[:40]) if len(tok) > 40 else float(tok)


def _case_blocks(body):
    """Split the body of a ``switch (sn)`` into {case_value: text}."""
    out = {}
    parts = re.split(r"\bcase\s+(\d+)\s*:", body)
    for i in range(1, len(parts), 2):
        out[int(parts[i])] = parts[i + 1]
    return out


def ls_tables(root):
    src = _strip_comments(_read(root, "src/LS.cc"))
    body = src[src.index("void LS::build_octant"):src.index("void LS::compute_omega")]
    tables = {}
    for sn, txt in _case_blocks(body).items():
        consts = {m.group(1): _eval_num(m.group(2), {})
                  for m in re.finditer(r"const double (w(?:_\d+)?)\(([-0-9.eE+/]+)\)", txt)}
        dirs = {int(m.group(1)): _num(m.group(2))
                for m in re.finditer(r"direction\[(\d+)\]\s*=\s*([-0-9.eE+]+)", txt)}
        if not dirs:  # S2 sets omega directly from a scalar
            m = re.search(r"const double direction\(([-0-9.eE+]+)\)", txt)
            dirs = {0: _num(m.group(1))}
        weights = {int(m.group(1)): m.group(2)
                   for m in re.finditer(r"weight\((\d+)\)\s*=\s*(w(?:_\d+)?)\s*;", txt)}
        n = len(weights)
        tables[str(sn)] = {
            "direction": [dirs[i] for i in range(len(dirs))],
            "weight": [consts[weights[i]] for i in range(n)],
            "weight_class": [weights[i] for i in range(n)],
        }
    return tables


def glc_gauss(root):
    src = _strip_comments(_read(root, "src/GLC.cc"))
    start = src.index("void GLC::build_gauss_legendre_quadrature")
    body = src[start:]
    out = {}
    for sn, txt in _case_blocks(body).items():
        nodes = {int(m.group(1)): _num(m.group(2))
                 for m in re.finditer(r"nodes\[(\d+)\]\s*=\s*([-0-9.eE+]+)", txt)}
        wts = {int(m.group(1)): _num(m.group(2))
               for m in re.finditer(r"weight\[(\d+)\]\s*=\s*([-0-9.eE+]+)", txt)}
        if nodes:
            out[str(sn)] = {"nodes": [nodes[i] for i in sorted(nodes)],
                            "weights": [wts[i] for i in sorted(wts)]}
    return out


def _inp(text):
    vals = {}
    for line in text.splitlines():
        m = re.match(r"\s*set\s+(.+?)\s*=\s*(.*?)\s*$", line)
        if m:
            vals[m.group(1)] = m.group(2)
    return vals


def rt_golden(root):
    src = _strip_comments(_read(root, "tests/RadiativeTransfer_test.cc"))
    sol = {int(m.group(1)): float(m.group(2))
           for m in re.finditer(r"solution\[(\d+)\]\s*=\s*([-0-9.eE+]+)", src)}
    tol = float(re.search(r"solution\[i\]\)\s*<\s*([0-9.eE+-]+)", src).group(1))
    return {
        "solution": [sol[i] for i in range(len(sol))],
        "tolerance": tol,
        "solver": "bicgstab" if "SolverBicgstab" in src else "gmres",
        "parameters": _inp(_read(root, "tests/rt_parameters.inp")),
        "geometry": _inp(_read(root, "tests/rt_geometry.inp")),
        "xs": _inp(_read(root, "tests/rt_xs.inp")),
        "dof_order": "deal.II hierarchical (z-order) cells, lexicographic local dofs",
    }


def quadrature_facts(root):
    src = _strip_comments(_read(root, "tests/RTQuadrature_test.cc"))
    ls_txt, glc_txt = src.split('TEST_CASE("RTQuadrature/GLC"')

    def common(txt):
        omega = [_num(m.group(2)) for m in
                 re.finditer(r"omega\[(\d)\]\s*=\s*([-0-9.eE+]+)\s*;", txt)]
        ctor = re.search(r"(LS|GLC) quad\((\d+),(\d+),(true|false)\)", txt)
        ls = {int(m.group(1)): int(m.group(2))
              for m in re.finditer(r"get_l\((\d+)\)==(\d+)", txt)}
        nd = re.search(r"unsigned int n_dir\((\d+)\)", txt)
        nm = re.search(r"unsigned int n_mom\((\d+)\)", txt)
        return {
            "type": ctor.group(1), "sn": int(ctor.group(2)), "L_max": int(ctor.group(3)),
            "galerkin": ctor.group(4) == "true",
            "weight_sum": "4pi", "dim": 2,
            "omega0": omega,
            "l": [ls[i] for i in range(len(ls))],
            "n_dir": int(nd.group(1)),
            "n_mom": int(nm.group(1)) if nm else int(nd.group(1)),
        }

    ls = common(ls_txt)
    mn = {}
    for m in re.finditer(r"is_most_normal_direction\((\d+),(\d+)\)==(true|false)", ls_txt):
        mn.setdefault(int(m.group(1)), {})[int(m.group(2))] = m.group(3) == "true"
    ls["most_normal"] = [[mn[f][d] for d in range(len(mn[f]))] for f in sorted(mn)]
    ls["omega0_exact"] = True
    glc = common(glc_txt)
    glc["omega0_exact"] = False
    return {"LS": ls, "GLC": glc}


# ----------------------------------------------------------------------------
# FECell test: a tiny interpreter for the statement forms the test uses.
# ----------------------------------------------------------------------------
def _split_statements(txt):
    """Tokenise into statements, '{', '}' and 'for' headers."""
    toks = []
    i, n = 0, len(txt)
    buf = ""
    while i < n:
        c = txt[i]
        if txt.startswith("for", i) and not buf.strip() and re.match(r"for\s*\(", txt[i:]):
            depth, j = 0, txt.index("(", i)
            k = j
            while True:
                if txt[k] == "(":
                    depth += 1
                elif txt[k] == ")":
                    depth -= 1
                    if depth == 0:
                        break
                k += 1
            toks.append(("for", txt[j + 1:k]))
            i = k + 1
            buf = ""
            continue
        if c in "{}":
            if buf.strip():
                toks.append(("stmt", buf.strip()))
            buf = ""
            toks.append((c, None))
        elif c == ";":
            toks.append(("stmt", buf.strip()))
            buf = ""
        else:
            buf += c
        i += 1
    return toks


def _parse_block(toks, pos):
    """Return (list_of_nodes, new_pos). Node: ('stmt', s) | ('for', hdr, body)."""
    nodes = []
    while pos < len(toks):
        kind, val = toks[pos]
        if kind == "}":
            return nodes, pos + 1
        node, pos = _parse_one(toks, pos)
        nodes.append(node)
    return nodes, pos


def _parse_one(toks, pos):
    kind, val = toks[pos]
    if kind == "{":
        body, pos = _parse_block(toks, pos + 1)
        return ("block", body), pos
    if kind == "for":
        body, pos = _parse_one(toks, pos + 1)
        return ("for", val, body), pos
    return ("stmt", val), pos + 1


def _eval_num(expr, env):
    expr = expr.strip()
    for k, v in env.items():
        expr = re.sub(r"\b%s\b" % k, repr(v), expr)
    expr = re.sub(r"(\d)\.(?!\d)", r"\1.0", expr)
    return float(eval(expr, {"__builtins__": {}}, {}))


def _run(nodes, env, state, out):
    for node in nodes:
        if node[0] == "block":
            _run(node[1], env, state, out)
        elif node[0] == "for":
            m = re.match(r"\s*unsigned int (\w+)\s*=\s*(\d+)\s*;\s*\1\s*<\s*(\d+)\s*;\s*\+\+\1\s*", node[1])
            var, lo, hi = m.group(1), int(m.group(2)), int(m.group(3))
            for v in range(lo, hi):
                env2 = dict(env)
                env2[var] = v
                _run([node[2]], env2, state, out)
        else:
            _stmt(node[1], env, state, out)


def _idx(tok, env):
    tok = tok.strip()
    return env[tok] if tok in env else int(tok)


def _stmt(s, env, state, out):
    s = " ".join(s.split())
    m = re.match(r"Tensor<2,\d+> (\w+)\(\*fecell\.get_(\w+)_matrix\((\w*)\)\)", s)
    if m is None:
        m = re.match(r"(\w+) = \*fecell\.get_(\w+)_matrix\((\w*)\)", s)
    if m:
        arg = m.group(3)
        state[m.group(1)] = (m.group(2), _idx(arg, env) if arg else None)
        return
    m = re.match(r"Point<2> const \* const (\w+) = fecell\.get_normal_vector\((\d+)\)", s)
    if m:
        state[m.group(1)] = ("normal", int(m.group(2)))
        return
    m = re.match(r"const double (\w+)\(([^)]*\)?)\)$", s)
    if m:
        env[m.group(1)] = _eval_num(m.group(2), env)
        return
    if not s.startswith("REQUIRE"):
        return
    inner = s[len("REQUIRE("):-1]
    m = re.match(r"(\w+)\[(\w+)\]\[(\w+)\]==0\.?$", inner)
    if m:
        kind, arg = state[m.group(1)]
        out.append({"matrix": kind, "arg": arg, "i": _idx(m.group(2), env),
                    "j": _idx(m.group(3), env), "value": 0.0, "exact": True})
        return
    m = re.match(r"std::fabs\((\w+)\[(\w+)\]\[(\w+)\](?:-\((.*)\))?\)<([0-9e.-]+)$", inner)
    if m:
        kind, arg = state[m.group(1)]
        val = _eval_num(m.group(4), env) if m.group(4) else 0.0
        out.append({"matrix": kind, "arg": arg, "i": _idx(m.group(2), env),
                    "j": _idx(m.group(3), env), "value": val, "exact": False,
                    "tol": float(m.group(5))})
        return
    m = re.match(r"std::fabs\(\(\*(\w+)\)\[(\d)\](?:-\(?([^()]*)\)?)?\)<([0-9e.-]+)$", inner)
    if m:
        kind, face = state[m.group(1)]
        val = _eval_num(m.group(3), env) if m.group(3) else 0.0
        out.append({"matrix": "normal", "arg": face, "i": int(m.group(2)), "j": None,
                    "value": val, "exact": False, "tol": float(m.group(4))})
        return
    m = re.match(r"fecell\.get_(material|source)_id\(\)==(\d+)$", inner)
    if m:
        out.append({"matrix": m.group(1) + "_id", "arg": None, "i": None, "j": None,
                    "value": float(m.group(2)), "exact": True})
        return
    raise ValueError("unparsed REQUIRE: " + s)


def fecell_facts(root):
    src = _strip_comments(_read(root, "tests/FECell_test.cc"))
    cases = re.split(r'TEST_CASE\("FECell/', src)[1:]
    out = {}
    for case in cases:
        name = case[:case.index('"')]
        body = case[case.index("{") + 1:]
        # mesh description used by the case
        mesh = {"fe_order": int(re.search(r"FE_DGQ<2> fe\((\d+)\)", body).group(1))}
        m = re.search(r"subdivided_hyper_cube\(triangulation,(\d+),([-0-9.]+),([-0-9.]+)\)", body)
        if m:
            mesh.update(subdivisions=int(m.group(1)), lo=float(m.group(2)), hi=float(m.group(3)))
        else:
            m = re.search(r"hyper_cube\(triangulation,([-0-9.]+),([-0-9.]+)\)", body)
            mesh.update(subdivisions=1, lo=float(m.group(1)), hi=float(m.group(2)))
        m = re.search(r"for \(unsigned int i=0; i<(\d+); \+\+i\)\s*\+\+cell;", body)
        mesh["cell"] = int(m.group(1)) if m else 0
        start = body.index("// Create the fecell") if "// Create the fecell" in case else 0
        toks = _split_statements(body[body.index("FECell<2,4> fecell"):])
        nodes, _ = _parse_block(toks, 0)
        facts = []
        _run(nodes, {}, {}, facts)
        out[name] = {"mesh": mesh, "facts": facts}
    return out


def inputs(root):
    names = ["geometry_2D.inp", "geometry_3D.inp", "rtmaterial_properties.inp",
             "parameters.inp", "rt_parameters.inp", "rt_geometry.inp", "rt_xs.inp"]
    files = {n: _read(root, "tests/" + n) for n in names}
    geo = _strip_comments(_read(root, "tests/Geometry_test.cc"))
    g2, g3 = geo.split('TEST_CASE("Geometry/3D"')

    def geo_expect(txt):
        sub = [int(m.group(2)) for m in re.finditer(r"get_n_subdivisions\((\d)\)==(\d+)", txt)]
        mats = [([int(x) for x in m.group(1).split(",")], int(m.group(2)))
                for m in re.finditer(r"get_material_ids\(([\d,]+)\)==(\d+)", txt)]
        srcs = [([int(x) for x in m.group(1).split(",")], int(m.group(2)))
                for m in re.finditer(r"get_source_ids\(([\d,]+)\)==(\d+)", txt)]
        nmat = int(re.search(r"get_n_materials\(\)==(\d+)", txt).group(1))
        return {"subdivisions": sub, "material_ids": mats, "source_ids": srcs, "n_materials": nmat}

    mat = _strip_comments(_read(root, "tests/RTMaterialProperties_test.cc"))
    st = [([int(x) for x in m.group(1).split(",")], float(m.group(2)))
          for m in re.finditer(r"get_sigma_t\(([\d,]+)\)==([0-9.]+)", mat)]
    ss = [([int(x) for x in m.group(1).split(",")], float(m.group(2)))
          for m in re.finditer(r"get_sigma_s\(([\d,]+)\)==([0-9.]+)", mat)]
    ctor = re.search(r"RTMaterialProperties mat_prop\(filename,(\d+),(\d+)\)", mat)
    prm = _strip_comments(_read(root, "tests/Parameters_test.cc"))
    pexp = []
    for m in re.finditer(r"REQUIRE\(parameters\.get_(\w+)\(([\d,]*)\)==(.+?)\);", prm):
        args = [int(x) for x in m.group(2).split(",")] if m.group(2) else []
        pexp.append([m.group(1), args, m.group(3).strip()])
    return {
        "files": files,
        "parameters": pexp,
        "geometry_2D": geo_expect(g2),
        "geometry_3D": geo_expect(g3),
        "materials": {"n_materials": int(ctor.group(1)), "n_groups": int(ctor.group(2)),
                      "sigma_t": st, "sigma_s": ss},
    }


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("OURANOS_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py <reference_root> (or set OURANOS_REFERENCE_ROOT)")
    outputs = {
        "ls_tables.json": ls_tables(root),
        "glc_gauss.json": glc_gauss(root),
        "rt_golden.json": rt_golden(root),
        "quadrature_facts.json": quadrature_facts(root),
        "fecell_facts.json": fecell_facts(root),
        "inputs.json": inputs(root),
    }
    for name, data in outputs.items():
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        print("wrote", name)


if __name__ == "__main__":
    main()

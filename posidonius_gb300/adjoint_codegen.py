"""Generator of the reverse-mode sweeps of the per-planet effect blocks.

The three additional-effect blocks of one planet -- constant-time-lag tides,
oblate rotational flattening, Kidder (1995) general relativity -- are
straight-line FP64 code.  This script restates them once (below, in the
FAST build's formulation of ``csrc/whfast_device.cuh``, which follows
src/effects/tides/constant_time_lag.rs:171-332, src/effects/tides/common.rs:
223-370, src/effects/rotational_flattening/oblate_spheroid.rs:12-97 and
src/effects/general_relativity.rs:177-456) by tracing them on a small
expression graph, and emits ``csrc/adjoint_effects.cuh``: for every block a
forward function and a vector-Jacobian product that recomputes the forward
values it needs and then runs the reverse sweep, adjoint by adjoint, in
registers.  Common subexpressions are merged and adjoints that nothing reads
are never formed.

Run ``python -m posidonius_gb300.adjoint_codegen`` after changing a block;
the generated header is committed.
"""
import os

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "csrc", "adjoint_effects.cuh")


class Node:
    __slots__ = ("op", "args", "val", "id", "name")

    def __init__(self, g, op, args=(), val=None, name=None):
        self.op, self.args, self.val, self.name = op, tuple(args), val, name
        self.id = None
        g._add(self)

    # arithmetic builds graph nodes
    def _g(self):
        return GRAPH

    def __add__(self, o):
        return GRAPH.op("add", self, o)

    def __radd__(self, o):
        return GRAPH.op("add", o, self)

    def __sub__(self, o):
        return GRAPH.op("sub", self, o)

    def __rsub__(self, o):
        return GRAPH.op("sub", o, self)

    def __mul__(self, o):
        return GRAPH.op("mul", self, o)

    def __rmul__(self, o):
        return GRAPH.op("mul", o, self)

    def __truediv__(self, o):
        return GRAPH.op("div", self, o)

    def __rtruediv__(self, o):
        return GRAPH.op("div", o, self)

    def __neg__(self):
        return GRAPH.op("neg", self)


class Graph:
    def __init__(self):
        self.nodes = []
        self.memo = {}
        self.inputs = []     # differentiable inputs (name)
        self.consts = []     # runtime constants (name), no adjoint

    def _add(self, n):
        n.id = len(self.nodes)
        self.nodes.append(n)

    def lit(self, v):
        key = ("lit", float(v))
        if key not in self.memo:
            self.memo[key] = Node(self, "lit", val=float(v))
        return self.memo[key]

    def inp(self, name):
        n = Node(self, "in", name=name)
        self.inputs.append(n)
        return n

    def const(self, name):
        n = Node(self, "cst", name=name)
        self.consts.append(n)
        return n

    def op(self, op, a, b=None):
        a = a if isinstance(a, Node) else self.lit(a)
        if b is not None:
            b = b if isinstance(b, Node) else self.lit(b)
        # constant folding of literal operands
        if a.op == "lit" and (b is None or b.op == "lit"):
            x, y = a.val, (b.val if b is not None else None)
            v = {"add": lambda: x + y, "sub": lambda: x - y, "mul": lambda: x * y, "div": lambda: x / y,
                 "neg": lambda: -x, "sqrt": lambda: x ** 0.5, "rcp": lambda: 1.0 / x}[op]()
            return self.lit(v)
        # a / b as a (1 / b): one division per divisor, shared by every
        # quotient and by the sweeps' derivatives (d(1/b) = -(1/b)^2 db)
        if op == "div":
            return self.op("mul", a, self.op("rcp", b))
        if op == "mul" and b is not None:
            if a.op == "lit" and a.val == 1.0:
                return b
            if b.op == "lit" and b.val == 1.0:
                return a
        args = (a,) if b is None else (a, b)
        if op in ("add", "mul"):  # commutative: canonical order for CSE
            args = tuple(sorted(args, key=lambda n: n.id))
        key = (op,) + tuple(n.id for n in args)
        if key not in self.memo:
            self.memo[key] = Node(self, op, args)
        return self.memo[key]


GRAPH = None


def sqrt(a):
    return GRAPH.op("sqrt", a)


def cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def powi(x, n):
    """x**n by square-and-multiply (n >= 1)."""
    result, base = None, x
    while n:
        if n & 1:
            result = base if result is None else result * base
        n >>= 1
        if n:
            base = base * base
    return result


# ---------------------------------------------------------------------------
# The blocks.  Inputs common to all: heliocentric position r = (x, y, z),
# heliocentric velocity hv, current spins S (planet) / H (host), previous
# spins P (planet) / Q (host) -- the r.Omega products of an evaluation use
# the spin of the previous evaluation.
# ---------------------------------------------------------------------------
K2 = "kK2"
C2 = "kC2"
FA = "kFA"
GLOBALS = {K2, C2, FA}  # compile-time constants of the device code

COMMON_INPUTS = ["x", "y", "z", "hv0", "hv1", "hv2", "S0", "S1", "S2", "H0", "H1", "H2",
                 "P0", "P1", "P2", "Q0", "Q1", "Q2"]


def _common(g):
    v = {n: g.inp(n) for n in COMMON_INPUTS}
    r = [v["x"], v["y"], v["z"]]
    hv = [v["hv0"], v["hv1"], v["hv2"]]
    S = [v["S0"], v["S1"], v["S2"]]
    H = [v["H0"], v["H1"], v["H2"]]
    P = [v["P0"], v["P1"], v["P2"]]
    Q = [v["Q0"], v["Q1"], v["Q2"]]
    d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2]
    d = sqrt(d2)
    return r, hv, S, H, P, Q, d


def block_tides(g):
    r, hv, S, H, P, Q, d = _common(g)
    sig_p, sig_h, k2_p, k2_h = g.inp("sig_p"), g.inp("sig_h"), g.inp("k2_p"), g.inp("k2_h")
    m, hm, R, hR = g.const("m"), g.const("hm"), g.const("R"), g.const("hR")
    inv_d = 1.0 / d
    rd = [c * inv_d for c in r]
    vr = dot(r, hv) * inv_d
    rs_s = dot(r, Q)
    rs_p = dot(r, P)
    h = cross(r, hv)
    d7 = powi(d, 7)
    d8 = d7 * d
    m2, hm2 = m * m, hm * hm
    term1 = m2 * powi(hR, 10) * sig_h
    term2 = hm2 * powi(R, 10) * sig_p
    o_s = 4.5 * term1 / d7
    o_p = 4.5 * term2 / d7
    cons = g.const(K2) * -3.0 / d7 * (m2 * powi(hR, 5) * k2_h + hm2 * powi(R, 5) * k2_p)
    osd, opd = o_s * inv_d, o_p * inv_d
    factor1 = vr * (-13.5 / d8)
    radial = cons + factor1 * (term1 + term2)
    factor3 = radial + (o_s + o_p) * inv_d * vr
    # osd (H x r - v) + opd (S x r - v) = (osd H + opd S) x r - (osd + opd) v
    w = [osd * H[k] + opd * S[k] for k in range(3)]
    wr = cross(w, r)
    ospd = (o_s + o_p) * inv_d
    F = [factor3 * rd[k] + wr[k] - ospd * hv[k] for k in range(3)]
    inv_m = 1.0 / m
    a = [inv_m * F[k] for k in range(3)]
    opdd, osdd = o_p * d, o_s * d
    qp, qs = o_p * rs_p, o_s * rs_s
    dl = [-(opdd * S[k] - qp * rd[k] - opd * h[k]) for k in range(3)]
    th = [-(osdd * H[k] - qs * rd[k] - osd * h[k]) for k in range(3)]
    return a + dl + th


def block_flat(g):
    r, hv, S, H, P, Q, d = _common(g)
    m, hm, R, hR = g.const("m"), g.const("hm"), g.const("R"), g.const("hR")
    k2f, hk2f = g.const("k2f"), g.const("hk2f")
    rs_s = dot(r, Q)
    rs_p = dot(r, P)
    cfs = m * hk2f * powi(hR, 5) * (1.0 / 6.0)
    cfp = hm * k2f * powi(R, 5) * (1.0 / 6.0)
    d5 = powi(d, 5)
    d7 = d5 * d * d
    inv_d5 = 1.0 / d5
    ofs = -6.0 * cfs * inv_d5 * rs_s
    ofp = -6.0 * cfp * inv_d5 * rs_p
    nsv2_p = dot(S, S)
    nsv2_h = dot(H, H)
    radial = (-3.0 / d5) * (cfp * nsv2_p + cfs * nsv2_h) + (15.0 / d7) * (cfs * rs_s * rs_s + cfp * rs_p * rs_p)
    F = [radial * r[k] + ofp * S[k] + ofs * H[k] for k in range(3)]
    inv_m = 1.0 / m
    a = [inv_m * F[k] for k in range(3)]
    rS, rH = cross(r, S), cross(r, H)
    dl = [-(ofp * rS[k]) for k in range(3)]
    th = [-(ofs * rH[k]) for k in range(3)]
    return a + dl + th


def block_gr(g):
    r, hv, S, H, P, Q, d = _common(g)
    m, hm, mg, hmg = g.const("m"), g.const("hm"), g.const("mg"), g.const("hmg")
    moi, hmoi = g.const("moi"), g.const("hmoi")
    c2 = g.const(C2)
    fa = g.const(FA)
    inv_d = 1.0 / d
    nn = [c * inv_d for c in r]
    vr = dot(r, hv) * inv_d
    nv2 = dot(hv, hv)
    mgs = hmg + mg
    f = hmg * mg / (mgs * mgs)
    d2 = d * d
    mgd = mgs * inv_d
    A = -mgs / (d2 * c2)
    B = 1.0 + 3.0 * f
    C = 2.0 * (2.0 + f) * mgd
    DD = 1.5 * f
    E = mgs / (d2 * c2) * 2.0 * (2.0 - f)
    T1 = 0.75 * (12.0 + 29.0 * f) * (mgs * mgs / d2)
    K2C = f * (3.0 - 4.0 * f)
    K3C = (15.0 / 8.0) * f * (1.0 - 3.0 * f)
    K4C = 1.5 * f * (3.0 - 4.0 * f)
    K5C = 0.5 * f * (13.0 - 4.0 * f) * mgd
    K6C = (2.0 + 25.0 * f + 2.0 * f * f) * mgd
    A05 = A * -0.5
    Pc = f * (15.0 + 4.0 * f)
    Qc = (4.0 + 41.0 * f + 8.0 * f * f) * mgd
    R3 = 3.0 * f * (3.0 + 2.0 * f)
    # the two orders as one polynomial in |v|^2 and v_r^2 (its coefficients
    # depend on the position only)
    GR0 = T1 - C
    GR1 = B - K5C
    GR2 = -(DD + K6C)
    GO0 = E - A05 * Qc
    GO1 = A05 * Pc
    GO2 = -(A05 * R3)
    vr2 = vr * vr
    rad = A * (GR0 + nv2 * (GR1 + K2C * nv2 - K4C * vr2) + vr2 * (GR2 + K3C * vr2))
    ort = vr * (GO0 + GO1 * nv2 + GO2 * vr2)
    gacc = [rad * nn[k] + ort * hv[k] for k in range(3)]
    # spin-orbit (general_relativity.rs:300-400, component-wise first term as
    # written there): ms = ((m_h - m) / M) M (L_p / m - L_h / m_h)
    sL = [hmoi * H[k] for k in range(3)]
    pL = [moi * S[k] for k in range(3)]
    mfm = hm - m
    ma, mb = mfm * moi / m, mfm / hm
    ms = [ma * S[k] - mb * sL[k] for k in range(3)]
    t = [sL[k] + pL[k] for k in range(3)]
    # (n x v)_k = (r x v)_k / d
    h = cross(r, hv)
    c6 = [6.0 * nn[k] * inv_d for k in range(3)]
    e1 = [c6[k] * (h[k] * (2.0 * t[k] + ms[k])) for k in range(3)]
    # -v x (7 t + 3 ms) + 3 v_r n x (3 t + ms) = aq x t + 3 q x ms with
    # q = v_r n - v, aq = 7 q + 2 v_r n
    q = [vr * nn[k] - hv[k] for k in range(3)]
    vr2x = 2.0 * vr
    aq = [7.0 * q[k] + vr2x * nn[k] for k in range(3)]
    axt = cross(aq, t)
    qxm = cross(q, ms)
    a = [gacc[k] + fa * (e1[k] + axt[k] + 3.0 * qxm[k]) for k in range(3)]
    # Kidder 1995 eq. 2.4a / 2.4b (general_relativity.rs:400-456): with
    # L_o = mu (r x v) the torques fm (L_o x S_h) - (L_p x S_h) + 3 (n.L_p) (n x S_h)
    # and fm2 (L_o x L_p) + (L_p x S_h) + 3 (n.S_h) (n x L_p), each one cross
    # product of a combined vector
    mu = hm * m / (hm + m)
    fmu = (2.0 + 1.5 * m / hm) * mu
    fm2mu = (2.0 + 1.5 * hm / m) * mu
    sp3 = 3.0 * dot(nn, pL)
    ss3 = 3.0 * dot(nn, sL)
    ws = [fmu * h[k] - pL[k] + sp3 * nn[k] for k in range(3)]
    wp = [fm2mu * h[k] - sL[k] + ss3 * nn[k] for k in range(3)]
    wsxs, wpxp = cross(ws, sL), cross(wp, pL)
    th = [fa * wsxs[k] for k in range(3)]
    dl = [fa * wpxp[k] for k in range(3)]
    return a + dl + th


OUTPUTS = ["a0", "a1", "a2", "dl0", "dl1", "dl2", "th0", "th1", "th2"]


# ---------------------------------------------------------------------------
# Emission
# ---------------------------------------------------------------------------
def _fmt(v):
    r = repr(float(v))
    return r if ("e" in r or "." in r or "n" in r) else r + ".0"


def _expr(n, names):
    a = [names[x.id] for x in n.args]
    if n.op == "add":
        return f"{a[0]} + {a[1]}"
    if n.op == "sub":
        return f"{a[0]} - {a[1]}"
    if n.op == "mul":
        return f"{a[0]} * {a[1]}"
    if n.op == "div":
        return f"{a[0]} / {a[1]}"
    if n.op == "rcp":
        return f"1.0 / {a[0]}"
    if n.op == "neg":
        return f"-{a[0]}"
    if n.op == "sqrt":
        return f"sqrt({a[0]})"
    raise ValueError(n.op)


def _live(outputs):
    """Nodes reachable from the outputs, in topological (creation) order."""
    seen = set()
    stack = list(outputs)
    while stack:
        n = stack.pop()
        if n.id in seen:
            continue
        seen.add(n.id)
        stack.extend(n.args)
    return seen


PRE_INPUTS = {"x", "y", "z", "sig_p", "sig_h", "k2_p", "k2_h"}


def emit(name, builder):
    """Emit, for one block, the split the midpoint loop needs: a 'pre' part
    (everything that depends only on the heliocentric position and the tidal
    parameters, fixed during a half kick) evaluated once per half kick, and an
    'iter' part evaluated per midpoint iteration from the pre values and the
    velocity / spin inputs; with the reverse sweeps of both (the iteration
    sweeps accumulate the adjoints of the pre values, which one pre sweep per
    half kick then takes back to the position and parameters)."""
    global GRAPH
    GRAPH = g = Graph()
    outs = builder(g)
    live = _live(outs)
    nodes = [n for n in g.nodes if n.id in live]
    inputs = list(g.inputs)
    consts = list(g.consts)
    names = {}
    for n in nodes:
        if n.op == "lit":
            names[n.id] = _fmt(n.val)
        elif n.op == "in":
            names[n.id] = f"in_{n.name}"
        elif n.op == "cst":
            names[n.id] = n.name if n.name in GLOBALS else f"c_{n.name}"
        else:
            names[n.id] = f"t{n.id}"
    grad = {}
    pre = {}
    for n in nodes:
        if n.op == "in":
            grad[n.id] = True
            pre[n.id] = n.name in PRE_INPUTS
        elif n.op in ("lit", "cst"):
            grad[n.id] = False
            pre[n.id] = True
        else:
            grad[n.id] = any(grad[a.id] for a in n.args)
            pre[n.id] = all(pre[a.id] for a in n.args)
    pre_in = [n for n in inputs if n.name in PRE_INPUTS]
    it_in = [n for n in inputs if n.name not in PRE_INPUTS]
    cst_names = sorted({n.name for n in consts if n.name not in GLOBALS})
    # pre values the iteration part reads (non-literal, non-constant pre nodes
    # used by iteration nodes or returned as outputs)
    it_nodes = [n for n in nodes if not pre[n.id]]
    pre_nodes = [n for n in nodes if pre[n.id] and n.op not in ("lit", "cst")]
    used = []
    seen = set()
    for n in it_nodes:
        for a in n.args:
            if pre[a.id] and a.op not in ("lit", "cst") and a.id not in seen:
                seen.add(a.id)
                used.append(a)
    for o in outs:
        if pre[o.id] and o.op not in ("lit", "cst") and o.id not in seen:
            seen.add(o.id)
            used.append(o)
    slot = {n.id: k for k, n in enumerate(used)}
    NPRE = len(used)
    sig_c = ", ".join(f"double c_{x}" for x in cst_names)
    sig_pre_in = ", ".join(f"double in_{n.name}" for n in pre_in)
    sig_it_in = ", ".join(f"double in_{n.name}" for n in it_in)
    L = []
    L.append(f"constexpr int {name}_NPRE = {NPRE};")
    L.append("")
    # ---- pre forward
    L.append(f"// {name}: values fixed during a half kick (position, tidal parameters).")
    L.append(f"__host__ __device__ __forceinline__ void {name}_pre({sig_pre_in},")
    L.append(f"        {sig_c}, double* __restrict__ pre) {{")
    for n in pre_nodes:
        if n.op == "in":
            continue
        L.append(f"    const double {names[n.id]} = {_expr(n, names)};")
    for n in used:
        L.append(f"    pre[{slot[n.id]}] = {names[n.id]};")
    L.append("}")
    L.append("")
    # ---- iteration forward
    def it_names():
        nm = dict(names)
        for n in used:
            nm[n.id] = f"pre[{slot[n.id]}]"
        return nm
    nm_it = it_names()
    it_fwd = [f"    const double {nm_it[n.id]} = {_expr(n, nm_it)};" for n in it_nodes if n.op != "in"]
    L.append(f"// {name}: one midpoint iteration.  Outputs: a[3] (planet acceleration),")
    L.append("// dl[3] (planet dL/dt), th[3] (dL/dt of the host due to this planet).")
    L.append(f"__host__ __device__ __forceinline__ void {name}_iter(const double* __restrict__ pre, {sig_it_in},")
    L.append(f"        {sig_c}, double* __restrict__ out) {{")
    L.extend(it_fwd)
    for k, o in enumerate(outs):
        L.append(f"    out[{k}] = {nm_it[o.id]};")
    L.append("}")
    L.append("")

    def reverse(node_list, nmap, seeds, boundary_pre):
        """Reverse sweep over node_list; contributions to pre values go to
        bpre[slot] when boundary_pre, else follow the nodes."""
        adj = {}
        body = []

        def contrib(n, term):
            if not grad[n.id] or n.op in ("lit", "cst"):
                return
            if boundary_pre and pre[n.id]:
                body.append(f"    bpre[{slot[n.id]}] += {term};")
                return
            if n.id in adj:
                body.append(f"    {adj[n.id]} += {term};")
            else:
                adj[n.id] = f"b{n.id}" if n.op != "in" else f"b_{n.name}"
                body.append(f"    double {adj[n.id]} = {term};")

        for n, term in seeds:
            contrib(n, term)
        for n in reversed(node_list):
            if n.op in ("lit", "in", "cst") or n.id not in adj:
                continue
            bn = adj[n.id]
            a = n.args
            an = [nmap[x.id] for x in a]
            if n.op == "add":
                contrib(a[0], bn)
                contrib(a[1], bn)
            elif n.op == "sub":
                contrib(a[0], bn)
                contrib(a[1], f"-{bn}")
            elif n.op == "neg":
                contrib(a[0], f"-{bn}")
            elif n.op == "mul":
                if a[0].id == a[1].id:
                    contrib(a[0], f"2.0 * {bn} * {an[0]}")
                else:
                    contrib(a[0], f"{bn} * {an[1]}")
                    contrib(a[1], f"{bn} * {an[0]}")
            elif n.op == "div":
                contrib(a[0], f"{bn} / {an[1]}")
                contrib(a[1], f"-{bn} * {nmap[n.id]} / {an[1]}")
            elif n.op == "rcp":
                contrib(a[0], f"-{bn} * {nmap[n.id]} * {nmap[n.id]}")
            elif n.op == "sqrt":
                contrib(a[0], f"0.5 * {bn} / {nmap[n.id]}")
        return body, adj

    # ---- iteration VJP
    seeds = [(o, f"bout[{k}]") for k, o in enumerate(outs)]
    body, adj = reverse(it_nodes, nm_it, seeds, True)
    L.append(f"// {name}: VJP of one iteration.  bin[{len(it_in)}] += adjoints of ({', '.join(n.name for n in it_in)});")
    L.append(f"// bpre[{name}_NPRE] += adjoints of the pre values.")
    L.append(f"__host__ __device__ __forceinline__ void {name}_iter_vjp(const double* __restrict__ pre, {sig_it_in},")
    L.append(f"        {sig_c}, const double* __restrict__ bout, double* __restrict__ bin, double* __restrict__ bpre) {{")
    L.extend(it_fwd)
    L.extend(body)
    for k, n in enumerate(it_in):
        if n.id in adj:
            L.append(f"    bin[{k}] += {adj[n.id]};")
    L.append("}")
    L.append("")
    # ---- pre VJP
    pre_fwd = [f"    const double {names[n.id]} = {_expr(n, names)};" for n in pre_nodes if n.op != "in"]
    seeds = [(n, f"bpre[{slot[n.id]}]") for n in used]
    body, adj = reverse(pre_nodes, names, seeds, False)
    L.append(f"// {name}: VJP of the pre values.  bin[{len(pre_in)}] += adjoints of ({', '.join(n.name for n in pre_in)}).")
    L.append(f"__host__ __device__ __forceinline__ void {name}_pre_vjp({sig_pre_in},")
    L.append(f"        {sig_c}, const double* __restrict__ bpre, double* __restrict__ bin) {{")
    L.extend(pre_fwd)
    L.extend(body)
    for k, n in enumerate(pre_in):
        if n.id in adj:
            L.append(f"    bin[{k}] += {adj[n.id]};")
    L.append("}")
    L.append("")
    return L, [n.name for n in pre_in], [n.name for n in it_in], cst_names, NPRE, len(it_fwd), len(body)


def emit_jvp(name, builder):
    """Forward-mode (tangent) versions of one block, for NT tangent directions
    (a template parameter): <block>_pre_jvp (values and tangents of the pre
    values) and <block>_iter_jvp (outputs and their tangents)."""
    global GRAPH
    GRAPH = g = Graph()
    outs = builder(g)
    live = _live(outs)
    nodes = [n for n in g.nodes if n.id in live]
    names = {}
    for n in nodes:
        if n.op == "lit":
            names[n.id] = _fmt(n.val)
        elif n.op == "in":
            names[n.id] = f"in_{n.name}"
        elif n.op == "cst":
            names[n.id] = n.name if n.name in GLOBALS else f"c_{n.name}"
        else:
            names[n.id] = f"t{n.id}"
    grad, pre = {}, {}
    for n in nodes:
        if n.op == "in":
            grad[n.id] = True
            pre[n.id] = n.name in PRE_INPUTS
        elif n.op in ("lit", "cst"):
            grad[n.id] = False
            pre[n.id] = True
        else:
            grad[n.id] = any(grad[a.id] for a in n.args)
            pre[n.id] = all(pre[a.id] for a in n.args)
    inputs, consts = list(g.inputs), list(g.consts)
    pre_in = [n for n in inputs if n.name in PRE_INPUTS]
    it_in = [n for n in inputs if n.name not in PRE_INPUTS]
    cst_names = sorted({n.name for n in consts if n.name not in GLOBALS})
    it_nodes = [n for n in nodes if not pre[n.id]]
    pre_nodes = [n for n in nodes if pre[n.id] and n.op not in ("lit", "cst")]
    used, seen = [], set()
    for n in it_nodes:
        for a in n.args:
            if pre[a.id] and a.op not in ("lit", "cst") and a.id not in seen:
                seen.add(a.id)
                used.append(a)
    for o in outs:
        if pre[o.id] and o.op not in ("lit", "cst") and o.id not in seen:
            seen.add(o.id)
            used.append(o)
    slot = {n.id: k for k, n in enumerate(used)}
    sig_c = ", ".join(f"double c_{x}" for x in cst_names)
    sig_pre_in = ", ".join(f"double in_{n.name}" for n in pre_in)
    sig_it_in = ", ".join(f"double in_{n.name}" for n in it_in)

    def tangent_lines(node_list, nm, dn):
        """dn(node) -> C expression of its tangent array element [k]."""
        L = []
        for n in node_list:
            if n.op in ("lit", "cst", "in") or not grad[n.id]:
                continue
            a = n.args
            an = [nm[x.id] for x in a]
            da = [dn(x) if grad[x.id] else None for x in a]
            if n.op == "add":
                e = " + ".join(d for d in da if d) or "0.0"
            elif n.op == "sub":
                e = da[0] if da[0] else ""
                if da[1]:
                    e = f"{e} - {da[1]}" if e else f"-{da[1]}"
            elif n.op == "neg":
                e = f"-{da[0]}"
            elif n.op == "mul":
                if a[0].id == a[1].id:
                    e = f"2.0 * {an[0]} * {da[0]}"
                else:
                    terms = []
                    if da[0]:
                        terms.append(f"{da[0]} * {an[1]}")
                    if da[1]:
                        terms.append(f"{an[0]} * {da[1]}")
                    e = " + ".join(terms)
            elif n.op == "div":
                if da[0] and da[1]:
                    e = f"({da[0]} - {nm[n.id]} * {da[1]}) / {an[1]}"
                elif da[0]:
                    e = f"{da[0]} / {an[1]}"
                else:
                    e = f"-{nm[n.id]} * {da[1]} / {an[1]}"
            elif n.op == "rcp":
                e = f"-{nm[n.id]} * {nm[n.id]} * {da[0]}"
            elif n.op == "sqrt":
                e = f"0.5 * {da[0]} / {nm[n.id]}"
            L.append(f"    double d{n.id}[NT];")
            L.append(f"#pragma unroll")
            L.append(f"    for (int k = 0; k < NT; ++k) d{n.id}[k] = {e};")
        return L

    out = []
    # ---- pre JVP
    out.append(f"// {name}: pre values and their tangents (din[i * NT + k]: tangent k of pre input i).")
    out.append("template <int NT>")
    out.append(f"__host__ __device__ __forceinline__ void {name}_pre_jvp({sig_pre_in},")
    out.append(f"        {sig_c}, const double* __restrict__ din, double* __restrict__ pre,")
    out.append("        double* __restrict__ dpre) {")
    for n in pre_nodes:
        if n.op != "in":
            out.append(f"    const double {names[n.id]} = {_expr(n, names)};")
    in_idx = {n.id: k for k, n in enumerate(pre_in)}

    def dn_pre(x):
        if x.op == "in":
            return f"din[{in_idx[x.id]} * NT + k]"
        return f"d{x.id}[k]"
    out.extend(tangent_lines(pre_nodes, names, dn_pre))
    for n in used:
        out.append(f"    pre[{slot[n.id]}] = {names[n.id]};")
        if grad[n.id]:
            out.append(f"#pragma unroll")
            out.append(f"    for (int k = 0; k < NT; ++k) dpre[{slot[n.id]} * NT + k] = {dn_pre(n)};")
        else:
            out.append(f"#pragma unroll")
            out.append(f"    for (int k = 0; k < NT; ++k) dpre[{slot[n.id]} * NT + k] = 0.0;")
    out.append("}")
    out.append("")
    # ---- iteration JVP
    nm = dict(names)
    for n in used:
        nm[n.id] = f"pre[{slot[n.id]}]"
    it_idx = {n.id: k for k, n in enumerate(it_in)}

    def dn_it(x):
        if x.id in slot:
            return f"dpre[{slot[x.id]} * NT + k]"
        if x.op == "in":
            return f"din[{it_idx[x.id]} * NT + k]"
        return f"d{x.id}[k]"
    out.append(f"// {name}: one iteration, outputs and their tangents (din[i * NT + k] for the")
    out.append(f"// iteration inputs; dout[o * NT + k]).")
    out.append("template <int NT>")
    out.append(f"__host__ __device__ __forceinline__ void {name}_iter_jvp(const double* __restrict__ pre,")
    out.append(f"        const double* __restrict__ dpre, {sig_it_in},")
    out.append(f"        {sig_c}, const double* __restrict__ din, double* __restrict__ out,")
    out.append("        double* __restrict__ dout) {")
    for n in it_nodes:
        if n.op != "in":
            out.append(f"    const double {nm[n.id]} = {_expr(n, nm)};")
    # grad of pre values used: they are grad if the pre node is grad
    out.extend(tangent_lines([n for n in it_nodes], nm, lambda x: dn_it(x) if (grad[x.id]) else None))
    for k_o, o in enumerate(outs):
        out.append(f"    out[{k_o}] = {nm[o.id]};")
        if grad[o.id]:
            out.append(f"#pragma unroll")
            out.append(f"    for (int k = 0; k < NT; ++k) dout[{k_o} * NT + k] = {dn_it(o)};")
        else:
            out.append(f"#pragma unroll")
            out.append(f"    for (int k = 0; k < NT; ++k) dout[{k_o} * NT + k] = 0.0;")
    out.append("}")
    out.append("")
    return out


def generate():
    blocks = [("adj_tides", block_tides), ("adj_flat", block_flat), ("adj_gr", block_gr)]
    out = ["// adjoint_effects.cuh -- GENERATED by posidonius_gb300/adjoint_codegen.py; do not edit.",
           "//",
           "// Per-planet additional-effect blocks (constant-time-lag tides, oblate",
           "// flattening, Kidder 1995 general relativity) in the formulation of the FAST",
           "// build, split for the implicit-midpoint loop: <block>_pre (once per half",
           "// kick: position and tidal-parameter terms), <block>_iter (per iteration),",
           "// the reverse sweeps <block>_iter_vjp / <block>_pre_vjp and the",
           "// forward-mode (tangent) sweeps <block>_pre_jvp / <block>_iter_jvp.",
           "#pragma once",
           "#include <cmath>",
           "",
           "#include \"adjoint_blocks.cuh\"",
           "",
           "namespace posi_adj {",
           ""]
    stats = []
    for name, fn in blocks:
        lines, pin, iin, csts, npre, nit, nrev = emit(name, fn)
        out.append(f"// {name}: pre inputs ({', '.join(pin)}); iteration inputs ({', '.join(iin)});")
        out.append(f"// constants ({', '.join(csts)})")
        out.extend(lines)
        out.extend(emit_jvp(name, fn))
        stats.append((name, npre, nit, nrev))
    out.append("}  // namespace posi_adj")
    out.append("")
    return "\n".join(out), stats


def main():
    text, stats = generate()
    with open(OUT, "w") as f:
        f.write(text)
    for name, npre, nit, nrev in stats:
        print(f"{name}: {npre} pre values, {nit} iteration statements, {nrev} pre-reverse statements")
    print(OUT)


if __name__ == "__main__":
    main()

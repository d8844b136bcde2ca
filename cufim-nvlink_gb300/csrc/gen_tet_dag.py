"""Generates tet_dag.inc: a level program that evaluates the FP64 prefix of
the reference's tet solve (solve_tet_cu, cuda_fim.h:1302-1360: the
coefficients b, c, e, the differences q13, q23, and sqt, pa, pb, sqt*X with
X = d*q13 - c*q23) on a group of lanes, one DFMA per lane and level.

Every operation of the prefix is a multiplication, addition or subtraction
of two doubles, and each is one correctly rounded DFMA with chosen operands:
    x * y = fma(x, y, -0.0)    x + y = fma(x, 1.0, y)    x - y = fma(x, 1.0, -y)
(x * 1.0 is exact; adding -0.0 leaves every product, signed zeros included,
as it is), and unary minus is a sign flip of an operand.  So evaluating the
expression tree of the source, node by node, in any order that respects its
dependences, gives exactly the values of the source's own evaluation (no
reassociation: the tree is the one C++ builds, left to right, unary minus
binding tightest).  Identical subexpressions are evaluated once.

The nodes are list-scheduled onto kDagLanes lanes, most critical path first.
Output: for every level and lane one word
    bits 0-7 slot of A, 8-15 slot of B, 16-23 slot of C,
    bits 24-26 sign flips of A, B, C
and the slots of the named results.  The node of level L and lane l writes
slot kDagLeaves + L * kDagLanes + l.

Usage: python gen_tet_dag.py  (rewrites tet_dag.inc beside this file)
"""
import os
import re

LANES = 8
# leaf slots (inputs and constants)
LEAVES = ["e13", "e23", "e34", "e12", "e14", "e24", "p1", "p2", "p3", "c0.5", "c2.0", "c1.0", "c-0.0"]
NLEAF = 16
ONE, NEGZERO = LEAVES.index("c1.0"), LEAVES.index("c-0.0")

# the prefix of solve_tet_cu as written in tet_ref (fim_device.cuh)
EXPRS = [
    ("a", "e13"),
    ("b", "0.5 * (e23 + e13 - e12)"),
    ("c", "-0.5 * (e34 + e13 - e14)"),
    ("d", "e23"),
    ("e", "-0.5 * (e34 + e23 - e24)"),
    ("f", "e34"),
    ("q13", "p3 - p1"),
    ("q23", "p3 - p2"),
    ("sqt", """-e*e*c*d*d + a*d*d*d*d - (b*b*c - a*c*c)*f*f + ((b*b - a*c)*f*f -
    (e*e*c - a*d*d - 2.*(e*c - b*d)*e)*f)*q13*q13 - 2.*(e*e*c*d -
    2.*e*b*d*d + a*d*d*d + (b*b - a*c)*d*f)*q13*q23 + (e*e*c*c -
    2.*e*b*c*d + a*c*d*d + (b*b*c - a*c*c)*f)*q23*q23 + 2.*(e*c*d*d -
    b*d*d*d)*e + (e*e*c*c + (b*b - 2.*a*c)*d*d - 2.*(e*c*c - b*c*d)*e)*f"""),
    ("pa", """e*c*d*d - b*d*d*d + (e*c - b*d)*f*q13*q13 - 2.*(e*c*d - b*d*d)*q13*q23 +
    (e*c*c - b*c*d)*q23*q23 - (e*c*c - b*c*d)*f"""),
    ("pb", """(d*d*d*d - 2.*c*d*d*f + c*c*f*f + (d*d*f - c*f*f)*q13*q13 -
    2.*(d*d*d - c*d*f)*q13*q23 + (c*d*d - c*c*f)*q23*q23)"""),
    ("X", "d*q13 - c*q23"),
    ("sx", "sqt*(d*q13 - c*q23)"),
]
OUTPUTS = ["b", "c", "e", "q13", "q23", "sqt", "pa", "pb", "X", "sx"]

_TOK = re.compile(r"\s*(?:(\d+\.\d*|\d+)|([A-Za-z_]\w*)|(\S))")


def _tokens(src):
    out = []
    for m in _TOK.finditer(src):
        if m.group(1):
            out.append(("num", float(m.group(1))))
        elif m.group(2):
            out.append(("id", m.group(2)))
        elif m.group(3):
            out.append(("op", m.group(3)))
    return out


class Dag:
    """Hash-consed expression DAG; a reference is (("leaf", slot) | ("node", i), negated)."""

    def __init__(self):
        self.nodes = []   # (op, ref_x, ref_y)
        self.memo = {}
        self.env = {}

    def node(self, op, x, y):
        key = (op, x, y)
        if key not in self.memo:
            self.memo[key] = ("node", len(self.nodes))
            self.nodes.append(key)
        return (self.memo[key], False)

    def parse(self, src):
        toks = _tokens(src)
        pos = [0]

        def peek():
            return toks[pos[0]] if pos[0] < len(toks) else (None, None)

        def take():
            t = peek()
            pos[0] += 1
            return t

        def primary():
            kind, val = take()
            if kind == "num":
                return (("leaf", LEAVES.index("c%r" % val)), False)
            if kind == "id":
                if val in self.env:
                    return self.env[val]
                return (("leaf", LEAVES.index(val)), False)
            if val != "(":
                raise SyntaxError(val)
            x = expr()
            if take() != ("op", ")"):
                raise SyntaxError("missing )")
            return x

        def unary():
            if peek() == ("op", "-"):
                take()
                r, neg = unary()
                return (r, not neg)
            return primary()

        def term():
            x = unary()
            while peek() == ("op", "*"):
                take()
                x = self.node("mul", x, unary())
            return x

        def expr():
            x = term()
            while peek() in (("op", "+"), ("op", "-")):
                op = "add" if take()[1] == "+" else "sub"
                x = self.node(op, x, term())
            return x

        r = expr()
        if pos[0] != len(toks):
            raise SyntaxError("trailing tokens in %r" % src)
        return r


def schedule(dag):
    users = [[] for _ in dag.nodes]
    for i, (_, x, y) in enumerate(dag.nodes):
        for r in (x, y):
            if r[0][0] == "node":
                users[r[0][1]].append(i)
    height = {}

    def hgt(i):
        if i not in height:
            height[i] = 1 + max((hgt(u) for u in users[i]), default=0)
        return height[i]

    place = {}
    level = 0
    while len(place) < len(dag.nodes):
        ready = [i for i in range(len(dag.nodes)) if i not in place and
                 all(r[0][0] == "leaf" or (r[0][1] in place and place[r[0][1]][0] < level)
                     for r in dag.nodes[i][1:])]
        ready.sort(key=lambda i: (-hgt(i), i))
        for lane, i in enumerate(ready[:LANES]):
            place[i] = (level, lane)
        level += 1
    return place, level


def main():
    dag = Dag()
    for name, src in EXPRS:
        dag.env[name] = dag.parse(src)
    place, levels = schedule(dag)

    def slot(ref):
        r, _ = ref
        if r[0] == "leaf":
            return r[1]
        lv, ln = place[r[1]]
        return NLEAF + lv * LANES + ln

    prog = [[0] * LANES for _ in range(levels)]
    for i, (op, x, y) in enumerate(dag.nodes):
        lv, ln = place[i]
        if op == "mul":
            a, b, c = slot(x), slot(y), NEGZERO
            flips = (x[1], y[1], False)
        else:
            a, b, c = slot(x), ONE, slot(y)
            flips = (x[1], False, y[1] != (op == "sub"))
        word = a | (b << 8) | (c << 16)
        for k, f in enumerate(flips):
            if f:
                word |= 1 << (24 + k)
        prog[lv][ln] = word
    out = {}
    for name in OUTPUTS:
        ref = dag.env[name]
        if ref[1]:
            raise ValueError("output %s is negated" % name)
        out[name] = slot(ref)
    nslots = NLEAF + levels * LANES
    if nslots > 256:
        raise ValueError("slots do not fit 8 bits")

    lines = [
        "// Generated by gen_tet_dag.py -- do not edit.  Level program of the FP64",
        "// prefix of solve_tet_cu (cuda_fim.h:1302-1360): %d DFMA nodes on %d lanes"
        % (len(dag.nodes), LANES),
        "// in %d levels (critical path %d)." % (levels, levels),
        "constexpr int kDagLanes = %d, kDagLevels = %d, kDagLeaves = %d;" % (LANES, levels, NLEAF),
        "constexpr int kDagSlots = kDagLeaves + kDagLevels * kDagLanes;",
        "// leaf slots: e13 e23 e34 e12 e14 e24 p1 p2 p3, then 0.5 2.0 1.0 -0.0",
        "constexpr int kDagLeafE13 = 0, kDagLeafP1 = 6, kDagLeafConst = 9;",
    ]
    lines.append("constexpr int " + ", ".join("kDagOut_%s = %d" % (n, out[n]) for n in OUTPUTS) + ";")
    lines.append("__constant__ uint32_t kTetDagProg[kDagLevels][kDagLanes] = {")
    for lv in range(levels):
        lines.append("  {" + ", ".join("0x%08xu" % w for w in prog[lv]) + "},")
    lines.append("};")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tet_dag.inc")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    print("%s: %d nodes, %d levels, %d slots" % (path, len(dag.nodes), levels, nslots))


if __name__ == "__main__":
    main()

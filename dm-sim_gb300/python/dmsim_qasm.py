"""OpenQASM 2.0 frontend: parse a QASM program straight into engine gates.

DM-Sim ships a translator that turns QASM into a generated Python script
(tool/dmsim_qasm.py, Python 2); this module parses the program and returns the
circuit (or appends it to a Simulation) directly.  Supported: the header and
``include "qelib1.inc";``, any number of ``qreg``/``creg`` (flattened in
declaration order), user ``gate`` definitions (expanded as macros, nested),
parameter expressions (numbers, ``pi``, + - * / ^, unary minus, sin cos tan exp
ln sqrt), register broadcast (``h q;`` applies to every qubit), ``barrier`` and
``measure`` (recorded, not simulated: measurement is ``Simulation.measure``).
``reset``, ``if`` and ``opaque`` raise ``QasmError``.

Gate names follow qelib1 and map onto DM-Sim's gate set with DM-Sim's
parameter slots (rz -> RZ(phi), crz/cu1/crx/cry -> lambda, rx/ry/rxx/rzz/ryy
-> theta).  ``u``/``U`` are U3, ``p`` is U1, ``cp`` is CU1.
"""
import ast
import math
import operator
import re

import dmsim_workloads as W

OP = W.OP


class QasmError(ValueError):
    pass


# name -> (DM-Sim op, number of qubits, parameter slots in QASM order)
GATES = {
    "u3": ("U3", 1, "tpl"), "u": ("U3", 1, "tpl"), "U": ("U3", 1, "tpl"), "u2": ("U2", 1, "pl"),
    "u1": ("U1", 1, "l"), "p": ("U1", 1, "l"), "cx": ("CX", 2, ""), "CX": ("CX", 2, ""), "id": ("ID", 1, ""),
    "x": ("X", 1, ""), "y": ("Y", 1, ""), "z": ("Z", 1, ""), "h": ("H", 1, ""), "s": ("S", 1, ""),
    "sdg": ("SDG", 1, ""), "t": ("T", 1, ""), "tdg": ("TDG", 1, ""), "rx": ("RX", 1, "t"), "ry": ("RY", 1, "t"),
    "rz": ("RZ", 1, "p"), "cz": ("CZ", 2, ""), "cy": ("CY", 2, ""), "swap": ("SWAP", 2, ""), "ch": ("CH", 2, ""),
    "ccx": ("CCX", 3, ""), "cswap": ("CSWAP", 3, ""), "crx": ("CRX", 2, "l"), "cry": ("CRY", 2, "l"),
    "crz": ("CRZ", 2, "l"), "cu1": ("CU1", 2, "l"), "cp": ("CU1", 2, "l"), "cu3": ("CU3", 2, "tpl"),
    "rxx": ("RXX", 2, "t"), "rzz": ("RZZ", 2, "t"), "ryy": ("RYY", 2, "t"), "rccx": ("RCCX", 3, ""),
    "rc3x": ("RC3X", 4, ""), "c3x": ("C3X", 4, ""), "c3sqrtx": ("C3SQRTX", 4, ""), "c4x": ("C4X", 5, ""),
}

_BIN = {ast.Add: operator.add, ast.Sub: operator.sub, ast.Mult: operator.mul, ast.Div: operator.truediv,
        ast.Pow: operator.pow}
_FUN = {"sin": math.sin, "cos": math.cos, "tan": math.tan, "exp": math.exp, "ln": math.log, "sqrt": math.sqrt}


def eval_param(expr, env=None):
    """Evaluate a QASM parameter expression (^ is power, as in QASM)."""
    env = env or {}
    try:
        # QASM's ^ is a power that binds tighter than * / and unary minus
        tree = ast.parse(expr.strip().replace("^", "**"), mode="eval")
    except SyntaxError as e:
        raise QasmError(f"bad parameter expression {expr!r}") from e

    def ev(node):
        if isinstance(node, ast.Expression):
            return ev(node.body)
        if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)):
            return float(node.value)
        if isinstance(node, ast.Name):
            if node.id == "pi":
                return math.pi
            if node.id in env:
                return env[node.id]
            raise QasmError(f"unknown name {node.id!r} in {expr!r}")
        if isinstance(node, ast.UnaryOp) and isinstance(node.op, (ast.USub, ast.UAdd)):
            v = ev(node.operand)
            return -v if isinstance(node.op, ast.USub) else v
        if isinstance(node, ast.BinOp) and type(node.op) in _BIN:
            return _BIN[type(node.op)](ev(node.left), ev(node.right))
        if isinstance(node, ast.Call) and isinstance(node.func, ast.Name) and node.func.id in _FUN and len(node.args) == 1:
            return _FUN[node.func.id](ev(node.args[0]))
        raise QasmError(f"unsupported expression {expr!r}")

    return ev(tree)


def _split_args(s):
    """Split on commas at parenthesis depth 0."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return [x.strip() for x in out]


_STMT = re.compile(r"^([A-Za-z_][A-Za-z0-9_]*)\s*(?:\((.*)\))?\s*(.*)$", re.S)


def parse_qasm(text, conditionals="error"):
    """Returns (n_qubits, circuit, measured) where circuit holds
    (op, qubits, theta, phi, lam) tuples for the engine.  A density matrix has
    no single measured outcome to branch on, so classically controlled
    statements (``if(c==k) ...;``) and ``reset`` raise QasmError, unless
    ``conditionals="skip"``: then they are dropped, gate included, as the
    reference's translator does (tool/dmsim_qasm.py:104, :321-322)."""
    if conditionals not in ("error", "skip"):
        raise ValueError("conditionals must be 'error' or 'skip'")
    text = re.sub(r"//[^\n]*", "", text)
    # gate definitions first (their bodies hold ';')
    gates = {}

    def take_gate_defs(src):
        out = ""
        i = 0
        pat = re.compile(r"\bgate\s+([A-Za-z_][A-Za-z0-9_]*)\s*(\(([^)]*)\))?\s*([^{]*)\{([^}]*)\}", re.S)
        for m in pat.finditer(src):
            out += src[i:m.start()]
            i = m.end()
            params = [p.strip() for p in (m.group(3) or "").split(",") if p.strip()]
            qargs = [q.strip() for q in m.group(4).split(",") if q.strip()]
            body = [b.strip() for b in m.group(5).split(";") if b.strip()]
            gates[m.group(1)] = (params, qargs, body)
        return out + src[i:]

    text = take_gate_defs(text)
    regs = {}
    nq = 0
    circuit = []
    measured = []

    def qubits_of(arg):
        arg = arg.strip()
        m = re.fullmatch(r"([A-Za-z_][A-Za-z0-9_]*)\s*\[\s*(\d+)\s*\]", arg)
        if m:
            name, idx = m.group(1), int(m.group(2))
            if name not in regs or idx >= regs[name][1]:
                raise QasmError(f"qubit {arg} out of range")
            return [regs[name][0] + idx]
        if arg in regs:
            off, size = regs[arg]
            return list(range(off, off + size))
        raise QasmError(f"unknown register {arg!r}")

    def emit(name, params, qubit_lists, depth=0):
        if depth > 64:
            raise QasmError("gate definitions nest too deeply")
        # broadcast: registers of equal length apply element-wise
        width = max(len(q) for q in qubit_lists) if qubit_lists else 1
        for qs in qubit_lists:
            if len(qs) not in (1, width):
                raise QasmError(f"register sizes do not match in {name}")
        for k in range(width):
            qs = [q[0] if len(q) == 1 else q[k] for q in qubit_lists]
            if name in gates:
                fparams, fq, body = gates[name]
                if len(fparams) != len(params) or len(fq) != len(qs):
                    raise QasmError(f"wrong arguments for gate {name}")
                env = dict(zip(fparams, params))
                qmap = dict(zip(fq, qs))
                for stmt in body:
                    m = _STMT.match(stmt)
                    if not m:
                        raise QasmError(f"bad statement {stmt!r} in gate {name}")
                    sub, sp, sq = m.group(1), m.group(2), m.group(3)
                    if sub == "barrier":
                        continue
                    subp = [eval_param(x, env) for x in _split_args(sp)] if sp else []
                    subq = [[qmap[a.strip()]] for a in sq.split(",") if a.strip()]
                    emit(sub, subp, subq, depth + 1)
            elif name in GATES:
                opname, ar, slots = GATES[name]
                if len(qs) != ar or len(params) != len(slots):
                    raise QasmError(f"gate {name} takes {ar} qubits and {len(slots)} parameters")
                if len(set(qs)) != len(qs):
                    raise QasmError(f"gate {name} repeats a qubit")
                vals = dict(zip(slots, params))
                circuit.append((OP[opname], tuple(qs), vals.get("t", 0.0), vals.get("p", 0.0), vals.get("l", 0.0)))
            else:
                raise QasmError(f"unknown gate {name!r}")

    for stmt in text.split(";"):
        stmt = stmt.strip()
        if not stmt:
            continue
        if stmt.startswith("OPENQASM") or stmt.startswith("include"):
            continue
        m = re.fullmatch(r"(qreg|creg)\s+([A-Za-z_][A-Za-z0-9_]*)\s*\[\s*(\d+)\s*\]", stmt)
        if m:
            if m.group(1) == "qreg":
                regs[m.group(2)] = (nq, int(m.group(3)))
                nq += int(m.group(3))
            continue
        if stmt.startswith("measure"):
            src = stmt[len("measure"):].split("->")[0]
            measured.extend(qubits_of(src))
            continue
        if conditionals == "skip" and (stmt.startswith("reset") or re.match(r"if\s*\(", stmt)):
            continue
        if stmt.startswith(("reset", "if", "opaque")):
            raise QasmError(f"unsupported statement: {stmt.split()[0]}")
        m = _STMT.match(stmt)
        if not m:
            raise QasmError(f"cannot parse {stmt!r}")
        name, ptxt, qtxt = m.group(1), m.group(2), m.group(3)
        if name == "barrier":
            continue
        params = [eval_param(x) for x in _split_args(ptxt)] if ptxt else []
        qlists = [qubits_of(a) for a in _split_args(qtxt)]
        emit(name, params, qlists)
    return nq, circuit, measured


def load_qasm(path_or_text, conditionals="error", **sim_options):
    """Parse a QASM file (or program text) into a new engine Simulation,
    uploaded and ready to run.  Returns (simulation, measured qubits)."""
    import dmsim_gb300 as E
    text = path_or_text
    if "\n" not in path_or_text and path_or_text.endswith(".qasm"):
        with open(path_or_text) as f:
            text = f.read()
    n, circ, measured = parse_qasm(text, conditionals=conditionals)
    sim = E.Simulation(n, **sim_options)
    sim.extend(circ)
    sim.upload()
    return sim, measured

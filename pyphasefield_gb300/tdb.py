"""Thermodynamic database (TDB) reader for the NCGPU engine.

pyphasefield builds its Gibbs energies with pycalphad (simulation.py:179-243,
ppf_utils.TDBContainer): per phase, the Redlich-Kister sum of the TDB's G
parameters plus the ideal mixing energy R T sum x ln x, components and phases
in sorted order. pycalphad is not a dependency here: this reader handles the
records such databases use (ELEMENT, PHASE, FUNCTION, PARAMETER G(phase,
component; 0) and the binary Redlich-Kister PARAMETER L(phase, A, B; k)) and
turns every temperature range of a pure element's Gibbs energy or of an
interaction parameter into coefficients of the basis

    1, T, T ln T, T^2, T^3, T^7, T^-1, T^-9

which the CUDA kernel evaluates per cell. An L parameter adds
x_A x_B L_k(T) (x_A - x_B)^k to its phase, A and B in the order the record
writes them (the CALPHAD convention for odd k). Sublattices and ternary
interactions are not read: a database that has them is rejected.
"""
from __future__ import annotations

import re
from pathlib import Path

BASIS = ("1", "T", "TLNT", "T2", "T3", "T7", "TM1", "TM9")
_POWER = {0: "1", 1: "T", 2: "T2", 3: "T3", 7: "T7", -1: "TM1", -9: "TM9"}
R_GAS = 8.3145  # pycalphad's gas constant, used in the ideal mixing energy

_NUM = r"[+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?"
# a number's mantissa and its exponent letter (1.5E, .5e), not a name that
# ends in E (GHSERFE): the sign that follows belongs to the exponent
_EXP_MANTISSA = re.compile(r"(?:^|[^A-Za-z_0-9.])(?:\d+\.?\d*|\.\d+)[eE]$")


class TdbError(ValueError):
    pass


def _split_terms(expr: str) -> list[str]:
    """Split at the top-level + and - signs (not inside parentheses, not in
    exponents like 1e-007)."""
    terms, depth, cur = [], 0, ""
    for i, ch in enumerate(expr):
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch in "+-" and depth == 0 and cur.strip() and not _EXP_MANTISSA.search(cur.strip()) \
                and not cur.rstrip().endswith("*"):
            terms.append(cur)
            cur = ch
        else:
            cur += ch
    if cur.strip():
        terms.append(cur)
    return [t.replace(" ", "") for t in terms]


def _term(term: str, functions: dict) -> tuple[dict, tuple | None]:
    """One term -> ({basis: coefficient}, None), or ({}, (sign, FUNCTION))
    for a reference to another FUNCTION."""
    sign = -1.0 if term.startswith("-") else 1.0
    body = term.lstrip("+-")
    if re.fullmatch(r"[A-Za-z_][A-Za-z_0-9]*", body) and body.upper() in functions:
        return {}, (sign, body.upper())
    coef, power, has_ln = sign, 0, False
    for f in body.upper().replace("**", "^").split("*"):
        if f == "LN(T)":
            has_ln = True
        elif f == "T":
            power += 1
        elif re.fullmatch(r"T\^\(?[+-]?\d+\)?", f):
            power += int(f[2:].strip("()"))
        elif re.fullmatch(_NUM, f):
            coef *= float(f)
        elif "/" in f and all(re.fullmatch(_NUM, q) for q in f.split("/")):
            q = f.split("/")
            coef *= float(q[0])
            for den in q[1:]:
                coef /= float(den)
        else:
            raise TdbError(f"unsupported TDB term {term!r}")
    if has_ln:
        if power != 1:
            raise TdbError(f"unsupported logarithmic term {term!r}")
        return {"TLNT": coef}, None
    if power not in _POWER:
        raise TdbError(f"unsupported power of T in {term!r}")
    return {_POWER[power]: coef}, None


class Database:
    """Pure-element Gibbs energies of an ideal-solution TDB."""

    def __init__(self, path):
        text = Path(path).read_text()
        lines = [ln.split("$", 1)[0] for ln in text.splitlines()]
        records = [r.strip() for r in " ".join(lines).split("!")]
        self.functions: dict[str, list] = {}
        raw_params: dict[tuple, list] = {}
        raw_excess: list[tuple] = []
        self.elements: list[str] = []
        self.phases: list[str] = []
        for rec in records:
            toks = rec.split()
            if not toks:
                continue
            kw = toks[0].upper()
            if kw in ("ELEMENT", "ELEM"):
                el = toks[1].upper()
                if el not in ("/-", "VA"):
                    self.elements.append(el)
            elif kw == "PHASE":
                # a phase name may carry a type suffix (LIQUID:L)
                self.phases.append(toks[1].upper().split(":")[0])
            elif kw in ("FUNCTION", "FUNCT", "FUNC"):
                self.functions[toks[1].upper()] = self._ranges(" ".join(toks[2:]))
            elif kw in ("PARAMETER", "PARAM", "PARA"):
                m = re.match(r"\S+\s+(\w)\s*\(\s*([^,]+?)\s*,\s*([^;]+?)\s*;\s*(\d+)\s*\)\s*(.*)",
                             rec)
                if not m:
                    raise TdbError(f"unreadable PARAMETER record {rec[:60]!r}")
                kind, phase, comp, order, body = m.groups()
                comps = [c.strip().upper() for c in comp.split(",")]
                if ":" in comp or any(not c for c in comps):
                    raise TdbError(f"sublattice parameters are not supported (got {rec[:60]!r})")
                if kind.upper() == "G" and int(order) == 0 and len(comps) == 1:
                    raw_params[(phase.upper(), comps[0])] = self._ranges(body)
                elif kind.upper() == "L" and len(comps) == 2:
                    raw_excess.append((phase.upper(), comps[0], comps[1], int(order),
                                       self._ranges(body)))
                else:
                    raise TdbError("only pure-element G and binary L parameters are supported "
                                   f"(got {rec[:60]!r})")
        self.elements.sort()
        self.phases.sort()
        self.params = {k: self._resolve(v) for k, v in raw_params.items()}
        # binary Redlich-Kister terms: (phase, A, B, order k, pieces)
        self.excess = [(ph, a, b, k, self._resolve(v)) for ph, a, b, k, v in raw_excess]
        for ph, a, b, k, _ in self.excess:
            if a not in self.elements or b not in self.elements or a == b:
                raise TdbError(f"L({ph},{a},{b};{k}): components must be two listed elements")

    @staticmethod
    def _ranges(body: str) -> list:
        parts = [p.strip() for p in body.split(";")]
        first = parts[0].split(None, 1)
        lo, expr = float(first[0]), first[1]
        out = []
        for p in parts[1:]:
            toks = p.split(None, 2)
            hi = float(toks[0])
            out.append((lo, hi, expr.strip()))
            if len(toks) == 3 and toks[1].upper() == "Y":
                lo, expr = hi, toks[2]
            else:
                break
        return out

    def _expand(self, expr: str, lo: float, hi: float, depth: int = 0) -> list:
        """[(T_lo, T_hi, {basis: coef})] for an expression valid on [lo, hi)."""
        if depth > 8:
            raise TdbError("FUNCTION references nest too deep")
        pieces = [(lo, hi, {})]
        # '#' marks a FUNCTION reference in some databases (GHSERNI#)
        for term in _split_terms(expr.replace("#", "")):
            coefs, ref = _term(term, self.functions)
            if ref is None:
                for _, _, acc in pieces:
                    for k, v in coefs.items():
                        acc[k] = acc.get(k, 0.0) + v
                continue
            sign, name = ref
            sub = []
            for flo, fhi, fexpr in self.functions[name]:
                sub.extend(self._expand(fexpr, flo, fhi, depth + 1))
            new = []
            for plo, phi_, acc in pieces:
                for slo, shi, sc in sub:
                    a, b = max(plo, slo), min(phi_, shi)
                    if a < b:
                        merged = dict(acc)
                        for k, v in sc.items():
                            merged[k] = merged.get(k, 0.0) + sign * v
                        new.append((a, b, merged))
            pieces = new
        return pieces

    def _resolve(self, ranges: list) -> list:
        out = []
        for lo, hi, expr in ranges:
            out.extend(self._expand(expr, lo, hi))
        return [(lo, hi, [c.get(b, 0.0) for b in BASIS]) for lo, hi, c in out]

    def scalar(self, name: str) -> float:
        """Constant FUNCTION value (evaluated at T = 1000, as pyphasefield's
        npvalue does, NCGPU.py:322-327)."""
        for lo, hi, expr in self.functions[name.upper()]:
            if lo <= 1000.0 < hi:
                pieces = self._expand(expr, lo, hi)
                return g_eval(pieces[0][2], 1000.0)
        return 0.0


def g_eval(coefs, T: float) -> float:
    import math
    c = coefs if isinstance(coefs, (list, tuple)) else [coefs.get(b, 0.0) for b in BASIS]
    return (c[0] + c[1] * T + c[2] * T * math.log(T) + c[3] * T ** 2 + c[4] * T ** 3
            + c[5] * T ** 7 + c[6] / T + c[7] * T ** -9)

"""Minimal symbolic algebra for boundary-class flux expressions.

Boundary classes (heatsim2's ``boundary_*`` protocol, doc/heatsim2_doc.xhtml "Defining boundary classes") are
Python callables ``qz/qy/qx(kmat_lo, kmat_hi, dz, dy, dx, <14 temperature placeholders>, *extra)`` that return
the face heat flux built from the placeholders with ``+ - * /``, indexing of the conductivity (``kmat[a,b]``)
and ``group(...)``.  ``group`` marks a difference that the Crank-Nicolson stage split treats as one unit
(heatsim2/expression.py:703-710 and crank_subst_in_groups :753-827 in the reference).

This module keeps the names ``linear_expression`` and ``group`` so the reference's boundary modules and user
classes written against them evaluate unchanged, but represents an expression as a sum of monomials
``coef * [k entry] * [T placeholder]`` with the group each T term belongs to -- enough to read off the face
conductance as an affine form in the conductivity entries (heatsim2_gb300.crank_nicolson compiles it).
Products are limited to degree one in k and degree one in T, which every aligned two-point flux satisfies.
"""
import itertools
import numbers

_group_ids = itertools.count(1)


class ExpressionError(ValueError):
    pass


class linear_expression(object):
    """A flux expression: {(k_name, k_index, T_name, group): coefficient}.

    ``linear_expression('kmat_lo')`` is a conductivity placeholder, ``linear_expression('Tp55')`` a temperature
    placeholder (names starting with ``kmat`` / ``T``), ``linear_expression(number)`` a constant.
    """

    __slots__ = ("terms",)

    def __init__(self, value=None):
        self.terms = {}
        if value is None:
            return
        if isinstance(value, linear_expression):
            self.terms = dict(value.terms)
        elif isinstance(value, numbers.Number):
            if value != 0:
                self.terms[(None, None, None, None)] = float(value)
        elif isinstance(value, str):
            if value.startswith("kmat"):
                self.terms[(value, None, None, None)] = 1.0
            elif value.startswith("T"):
                self.terms[(None, None, value, None)] = 1.0
            else:
                raise ExpressionError("unknown placeholder %r" % (value,))
        else:
            raise ExpressionError("cannot build an expression from %r" % (type(value),))

    # -- construction helpers ---------------------------------------------------------------------------
    @staticmethod
    def _coerce(v):
        if isinstance(v, linear_expression):
            return v
        if isinstance(v, numbers.Number):
            return linear_expression(v)
        raise ExpressionError("unsupported operand %r" % (type(v),))

    def _add_terms(self, other, sign):
        res = linear_expression(self)
        for key, c in other.terms.items():
            res.terms[key] = res.terms.get(key, 0.0) + sign * c
        return res

    def _scaled(self, s):
        res = linear_expression()
        res.terms = {key: c * s for key, c in self.terms.items()}
        return res

    # -- arithmetic -------------------------------------------------------------------------------------
    def __add__(self, other):
        return self._add_terms(self._coerce(other), 1.0)

    def __radd__(self, other):
        return self._coerce(other)._add_terms(self, 1.0)

    def __sub__(self, other):
        return self._add_terms(self._coerce(other), -1.0)

    def __rsub__(self, other):
        return self._coerce(other)._add_terms(self, -1.0)

    def __neg__(self):
        return self._scaled(-1.0)

    def __pos__(self):
        return linear_expression(self)

    def __mul__(self, other):
        if isinstance(other, numbers.Number):
            return self._scaled(float(other))
        other = self._coerce(other)
        res = linear_expression()
        for (k1, i1, t1, g1), c1 in self.terms.items():
            for (k2, i2, t2, g2), c2 in other.terms.items():
                if k1 is not None and k2 is not None:
                    raise ExpressionError("product of two conductivities: flux is not linear in k")
                if t1 is not None and t2 is not None:
                    raise ExpressionError("product of two temperatures: flux is not linear in T")
                key = (k1 if k1 is not None else k2, i1 if k1 is not None else i2,
                       t1 if t1 is not None else t2, g1 if t1 is not None else g2)
                res.terms[key] = res.terms.get(key, 0.0) + c1 * c2
        return res

    __rmul__ = __mul__

    def __truediv__(self, other):
        if isinstance(other, linear_expression):
            if set(other.terms) - {(None, None, None, None)}:
                raise ExpressionError("division by a non-constant expression")
            other = other.terms.get((None, None, None, None), 0.0)
        if not isinstance(other, numbers.Number):
            raise ExpressionError("unsupported divisor %r" % (type(other),))
        res = linear_expression()
        res.terms = {key: c / float(other) for key, c in self.terms.items()}
        return res

    def __rtruediv__(self, other):
        raise ExpressionError("division by an expression")

    def __getitem__(self, index):
        """Index the conductivity placeholders of this expression, e.g. ``kmat[0, 0]`` (z,y,x order)."""
        if not (isinstance(index, tuple) and len(index) == 2):
            raise ExpressionError("conductivity index must be a pair (row, column)")
        r, c = int(index[0]), int(index[1])
        if not (0 <= r < 3 and 0 <= c < 3):
            raise ExpressionError("conductivity index %r outside 3x3" % (index,))
        res = linear_expression()
        for (k, i, t, g), coef in self.terms.items():
            if t is not None and k is None:
                raise ExpressionError("indexing a temperature")
            key = (k, (r, c) if (k is not None and i is None) else i, t, g)
            res.terms[key] = res.terms.get(key, 0.0) + coef
        return res

    # -- inspection -------------------------------------------------------------------------------------
    def temperature_terms(self):
        """{(T_name, group): [(k_name, k_index, coef), ...]} for the T-dependent part."""
        out = {}
        for (k, i, t, g), c in self.terms.items():
            if t is not None:
                out.setdefault((t, g), []).append((k, i, c))
        return out

    def constant_terms(self):
        return [(k, i, c) for (k, i, t, g), c in self.terms.items() if t is None]

    def __repr__(self):
        parts = []
        for (k, i, t, g), c in sorted(self.terms.items(), key=lambda kv: str(kv[0])):
            s = "%.17g" % c
            if k is not None:
                s += "*%s%s" % (k, "" if i is None else "[%d,%d]" % i)
            if t is not None:
                s += "*%s" % t
            if g is not None:
                s += "{g%d}" % g
            parts.append(s)
        return "linear_expression(%s)" % (" + ".join(parts) if parts else "0")


def group(expr):
    """Mark the temperature terms of ``expr`` as one Crank-Nicolson unit (reference expression.py:703-710).
    An outer group replaces inner ones, as the reference's group scan finds the outermost group first."""
    expr = linear_expression._coerce(expr)
    gid = next(_group_ids)
    res = linear_expression()
    for (k, i, t, g), c in expr.terms.items():
        key = (k, i, t, gid if t is not None else g)
        res.terms[key] = res.terms.get(key, 0.0) + c
    return res

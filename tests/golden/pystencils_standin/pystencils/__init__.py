"""Test-only stand-in for the part of pystencils 1.x that the reference's
``pyaxisymflow/pyst_kernels`` modules use, so that those modules run
unmodified and their own symbolic kernels can be evaluated here.

TEST INFRASTRUCTURE ONLY (pystencils is not installed in this environment).
It restates pystencils' published semantics for this subset:

* ``fields("a, b : float64[2D]")`` / ``[n0, n1]``: fields whose relative
  accesses ``f[i, j]`` are sympy symbols named ``f_<direction>`` as pystencils
  names them (``offset_to_direction_string``: axis 0 is x = East/West, axis 1
  is y = North/South, magnitudes above one as a prefix, ``C`` for the centre),
  so sympy orders sums and products of them as it does under pystencils;
* ``@kernel``: the decorated function's source is re-parsed, ``lhs @= rhs``
  becomes an assignment and ``a if c else b`` becomes
  ``sympy.Piecewise((a, c), (b, True))``;
* ``create_kernel(assignments, config=...).compile()``: a callable taking the
  fields and symbols by keyword. It updates every cell at least ``g`` cells
  from every edge, ``g`` being the largest access offset of the kernel
  (pystencils' automatic ghost-layer rule with ``ghost_layers=None``).
  Each right-hand side is printed by sympy's C code printer, which fixes the
  order of the terms of every sum and the factors of every product and prints
  the constants with 17 significant digits; the printed expression is then
  evaluated over numpy slices in IEEE double precision, left to right, with
  no contraction into fused multiply-adds.

What it does not model: pystencils compiles the printed C with its own
compiler flags (by default an optimising, fast-math configuration), which may
reassociate or contract the arithmetic; the evaluation here is the printed
expression taken literally.
"""
import ast
import inspect
import textwrap

import numpy as np
import sympy as sp
from sympy.printing.c import C89CodePrinter

__all__ = ["CreateKernelConfig", "fields", "kernel", "create_kernel", "Assignment"]


class CreateKernelConfig:
    def __init__(self, data_type="float64", default_number_float="float64", cpu_openmp=False,
                 **kwargs):
        if data_type != "float64":
            raise NotImplementedError("the stand-in evaluates float64 kernels only")
        self.data_type = data_type
        self.default_number_float = default_number_float
        self.cpu_openmp = cpu_openmp
        self.extra = kwargs


def offset_to_direction_string(offsets):
    """Direction name of an access offset: x (axis 0) East / West, y (axis 1)
    North / South, z Top / Bottom, last axis first, magnitude > 1 as a prefix."""
    names = ("E", "W", "N", "S", "T", "B")
    out = ""
    for ax in range(len(offsets) - 1, -1, -1):
        o = int(offsets[ax])
        if o == 0:
            continue
        if abs(o) > 1:
            out += str(abs(o))
        out += names[2 * ax] if o > 0 else names[2 * ax + 1]
    return out or "C"


class Access(sp.Symbol):
    """A relative access ``field[offsets]`` (a sympy symbol)."""

    def __new__(cls, field_name, offsets):
        obj = super().__new__(cls, f"{field_name}_{offset_to_direction_string(offsets)}")
        obj.field_name = field_name
        obj.offsets = tuple(int(o) for o in offsets)
        return obj


class Field:
    def __init__(self, name, dtype, shape):
        self.name = name
        self.dtype = dtype
        self.shape = shape  # None: any 2-D shape

    def __getitem__(self, idx):
        idx = idx if isinstance(idx, tuple) else (idx,)
        return Access(self.name, idx)


def fields(spec):
    """``"a, b, c : float64[2D]"`` or ``"... : float64[512, 256]"``."""
    names, typ = spec.split(":")
    dtype, dims = typ.strip().split("[")
    dims = dims.rstrip("]").strip()
    if dims.endswith("D"):
        shape = None
        if int(dims[:-1]) != 2:
            raise NotImplementedError("the stand-in handles 2-D fields")
    else:
        shape = tuple(int(x) for x in dims.split(","))
        if len(shape) != 2:
            raise NotImplementedError("the stand-in handles 2-D fields")
    out = [Field(n.strip(), dtype.strip(), shape) for n in names.split(",")]
    return out[0] if len(out) == 1 else tuple(out)


class Assignment:
    def __init__(self, lhs, rhs):
        self.lhs = lhs
        self.rhs = sp.sympify(rhs)


class _KernelRewrite(ast.NodeTransformer):
    """``lhs @= rhs`` -> ``_add_assignment(lhs, rhs)``;
    ``a if c else b`` -> ``_Piecewise((a, c), (b, True))``."""

    def visit_FunctionDef(self, node):
        node.decorator_list = []
        self.generic_visit(node)
        return node

    def visit_IfExp(self, node):
        self.generic_visit(node)
        call = ast.Call(func=ast.Name(id="_Piecewise", ctx=ast.Load()),
                        args=[ast.Tuple(elts=[node.body, node.test], ctx=ast.Load()),
                              ast.Tuple(elts=[node.orelse, ast.Constant(value=True)],
                                        ctx=ast.Load())],
                        keywords=[])
        return ast.copy_location(call, node)

    def visit_AugAssign(self, node):
        self.generic_visit(node)
        if not isinstance(node.op, ast.MatMult):
            return node
        target = node.target
        target.ctx = ast.Load()
        call = ast.Call(func=ast.Name(id="_add_assignment", ctx=ast.Load()),
                        args=[target, node.value], keywords=[])
        return ast.copy_location(ast.Expr(value=call), node)


def kernel(func):
    """Collect the assignments of a kernel function (pystencils' @kernel)."""
    tree = ast.parse(textwrap.dedent(inspect.getsource(func)))
    tree = _KernelRewrite().visit(tree)
    ast.fix_missing_locations(tree)
    assignments = []
    scope = dict(func.__globals__)
    scope.update(inspect.getclosurevars(func).nonlocals)
    scope["_add_assignment"] = lambda lhs, rhs: assignments.append(Assignment(lhs, rhs))
    scope["_Piecewise"] = sp.Piecewise
    exec(compile(tree, "<pystencils stand-in kernel>", "exec"), scope)
    scope[func.__name__]()
    return assignments


class _SlicePrinter(C89CodePrinter):
    """sympy's C printer (term and factor order, 17-digit constants) with
    conditionals printed as numpy selections."""

    def _print_Piecewise(self, expr):
        if len(expr.args) != 2 or expr.args[1].cond != sp.true:
            raise NotImplementedError("two-branch conditionals only")
        (a, c), (b, _) = expr.args
        return f"_where({self._print(c)}, {self._print(a)}, {self._print(b)})"


def _accesses(expr):
    return {s for s in expr.free_symbols if isinstance(s, Access)}


class _Compiled:
    def __init__(self, assignments):
        self.assignments = assignments
        acc = set()
        for a in assignments:
            acc |= _accesses(a.rhs) | {a.lhs}
        self.ghost = max(max(abs(o) for o in s.offsets) for s in acc)
        printer = _SlicePrinter()
        self.code = [(a.lhs, compile(printer.doprint(a.rhs), "<stand-in rhs>", "eval"),
                      sorted(_accesses(a.rhs), key=lambda s: s.name),
                      sorted((s for s in a.rhs.free_symbols if not isinstance(s, Access)),
                             key=lambda s: s.name))
                     for a in assignments]
        self.printed = [printer.doprint(a.rhs) for a in assignments]

    def __call__(self, **kwargs):
        g = self.ghost
        for lhs, code, accs, syms in self.code:
            out = kwargs[lhs.field_name]
            if out.dtype != np.float64 or out.ndim != 2:
                raise TypeError("the stand-in evaluates 2-D float64 fields")
            n0, n1 = out.shape
            env = {"_where": np.where}
            for s in accs:
                arr = kwargs[s.field_name]
                if arr.shape != out.shape:
                    raise ValueError("fields of one kernel must have the same shape")
                o0, o1 = s.offsets
                env[s.name] = arr[g + o0:n0 - g + o0, g + o1:n1 - g + o1]
            for s in syms:
                env[s.name] = np.float64(kwargs[s.name])
            val = eval(code, env)
            out[g:n0 - g, g:n1 - g] = val


class _KernelAst:
    def __init__(self, assignments, config):
        self.assignments = assignments
        self.config = config

    def compile(self):
        return _Compiled(self.assignments)


def create_kernel(assignments, config=None, **kwargs):
    if not isinstance(assignments, (list, tuple)):
        assignments = [assignments]
    return _KernelAst(list(assignments), config)

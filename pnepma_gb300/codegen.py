"""Emit the per-order stencil header used by the CUDA kernels.

For every compiled P_N order the header holds, per class c and axis d, the sparsity of the
advection block ``A_d[c]`` as straight-line code in column-major (CSC) order: for each column j
the difference ``f(j)`` of the neighbouring from-class values is formed once and scattered into
the rows that couple to it.  This is the traversal of ``matmuldiff!`` for a sparse block
(``starmap/src/solver_core.jl:59-69``); the row accumulation order is therefore the reference's.

Coefficients come from a functor ``coef(k, literal)``: the FP64 single-solve path reads them from
a per-solve table already divided by the grid step, the FP32 batched path uses the literal value.
Run as a module to regenerate the header:  ``python -m pnepma_gb300.codegen``.
"""
from __future__ import annotations

import os
import sys

from .matrices import advection_block
from .moments import N_CLASSES, class_moments, switch

ORDERS = (1, 3, 5, 7, 9, 11)
HEADER = os.path.join(os.path.dirname(__file__), "csrc", "generated", "pn_stencils.cuh")


def block_structure(N: int, c: int, d: int):
    """CSC traversal of A_d[c]: list of (col, [(row, value), ...]) for non-empty columns."""
    A = advection_block(N, c, d)
    cols = []
    for j in range(A.shape[1]):
        rows = [(i, float(A[i, j])) for i in range(A.shape[0]) if A[i, j] != 0.0]
        if rows:
            cols.append((j, rows))
    return cols


def table_layout(N: int):
    """Offsets of each (class, axis) block in the flat nnz table and the total size."""
    off = {}
    k = 0
    for c in range(N_CLASSES):
        for d in range(3):
            off[(c, d)] = k
            k += sum(len(r) for _j, r in block_structure(N, c, d))
    return off, k


def _lit(v: float) -> str:
    return repr(float(v))


def emit(orders=ORDERS) -> str:
    out = []
    w = out.append
    w("// Generated by pnepma_gb300/codegen.py -- do not edit.")
    w("// Sparse advection stencils per P_N order, class and axis (CSC traversal order).")
    w("#pragma once")
    w("")
    w("namespace pn {")
    w("")
    w("template <int N> struct Ord;")
    w("")
    for N in orders:
        ms = class_moments(N)
        n = [len(v) for v in ms]
        maxn = max(n)
        off, total = table_layout(N)
        w(f"template <> struct Ord<{N}> {{")
        w(f"  static constexpr int N = {N};")
        w(f"  static constexpr int maxn = {maxn};")
        w(f"  static constexpr int n_tab = {total};")
        w(f"  static __host__ __device__ constexpr int n(int c) {{ return " +
          " ".join(f"c == {c} ? {n[c]} :" for c in range(7)) + f" {n[7]}; }}")
        # degree of each moment
        for c in range(N_CLASSES):
            degs = [l for (l, _k) in ms[c]] or [0]
            w(f"  static constexpr int deg{c}[{max(1, len(degs))}] = {{{', '.join(map(str, degs))}}};")
        cases = []
        for c in range(N_CLASSES):
            for m, (l, _k) in enumerate(ms[c]):
                cases.append(f"case {c * 64 + m}: return {l};")
        w("  static __host__ __device__ constexpr int deg(int c, int m) {")
        w("    switch (c * 64 + m) { " + " ".join(cases) + " default: return 0; }")
        w("  }")
        masks = []
        for c in range(N_CLASSES):
            mk = 0
            for (l, _k) in ms[c]:
                mk |= 1 << l
            masks.append(mk)
        w(f"  static __host__ __device__ constexpr unsigned deg_mask(int c) {{ return " +
          " ".join(f"c == {c} ? {masks[c]}u :" for c in range(7)) + f" {masks[7]}u; }}")
        rc = []
        for c in range(N_CLASSES):
            for d in range(3):
                for j, rows in block_structure(N, c, d):
                    for (i, _v) in rows:
                        rc.append(f"{{{i}, {j}}}")
        vals = []
        for c in range(N_CLASSES):
            for d in range(3):
                for j, rows in block_structure(N, c, d):
                    for (i, v) in rows:
                        vals.append(_lit(v))
        w(f"  // closed-form value of every table entry, in table order")
        w(f"  static constexpr double val[{max(1, len(vals))}] = {{{', '.join(vals) if vals else '0.0'}}};")
        w(f"  // (row, column) of every table entry, in table order")
        w(f"  static constexpr short rc[{max(1, len(rc))}][2] = {{{', '.join(rc) if rc else '{0, 0}'}}};")
        w(f"  static __host__ __device__ constexpr int off(int c, int d) {{ return " +
          " ".join(f"(c == {c} && d == {d}) ? {off[(c, d)]} :" for c in range(N_CLASSES) for d in range(3)) +
          " 0; }")
        w("};")
        w("")
    # degree accessor
    w("template <int N, int C> __host__ __device__ constexpr int degree_of(int m) { return Ord<N>::deg(C, m); }")
    w("")
    w("template <int N, int C, int D> struct Adv;")
    w("")
    for N in orders:
        for c in range(N_CLASSES):
            for d in range(3):
                cols = block_structure(N, c, d)
                nf = len(class_moments(N)[switch(c, d)])
                w(f"template <> struct Adv<{N}, {c}, {d}> {{")
                w(f"  static constexpr int n_from = {nf};")
                w(f"  static constexpr int nnz = {sum(len(r) for _j, r in cols)};")
                w("  template <class T, class Acc, class Diff, class Coef>")
                w("  __device__ __forceinline__ static void apply(Acc& acc, const Diff& f, const Coef& coef) {")
                k = 0
                for j, rows in cols:
                    w(f"    {{ const T v = f({j});")
                    for (i, val) in rows:
                        w(f"      acc[{i}] = fma(coef({k}, {_lit(val)}), v, acc[{i}]);")
                        k += 1
                    w("    }")
                if not cols:
                    w("    (void)acc; (void)f; (void)coef;")
                w("  }")
                w("};")
        w("")
    w("}  // namespace pn")
    w("")
    return "\n".join(out)


def emit_orders(orders=ORDERS) -> str:
    return ("// Generated by pnepma_gb300/codegen.py -- do not edit.\n#pragma once\n"
            "#define PN_FOR_EACH_ORDER(X) " + " ".join(f"X({N})" for N in orders) + "\n")


def _write_if_changed(path: str, text: str) -> None:
    old = None
    if os.path.exists(path):
        with open(path) as fh:
            old = fh.read()
    if old != text:
        with open(path, "w") as fh:
            fh.write(text)


def write_header(path: str = HEADER, orders=ORDERS) -> str:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    _write_if_changed(path, emit(orders))
    _write_if_changed(os.path.join(os.path.dirname(path), "pn_orders.h"), emit_orders(orders))
    return path


if __name__ == "__main__":
    print(write_header(), file=sys.stderr)

"""Restatement of the reference's print_tree (Parallel/RustVersion/src/array_kd_tree.rs:666-692)
for checking the library's dump: first line tree.len(), then per slot "L n" + "x y z" lines or
"I split_dim split_val left right", numbers as Rust's `{}` prints f64."""
from __future__ import annotations

import math
from decimal import Decimal


def rust_f64(x: float) -> str:
    """Rust's Display for f64: shortest round-trip digits, positional notation."""
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    s = format(Decimal(repr(x)), "f")
    if "." in s:
        s = s.rstrip("0").rstrip(".")
    return s


def print_tree(nodes, bodies, length: int) -> str:
    out = [f"{length}"]
    for i in range(length):
        if i >= len(nodes):
            out.append("L 0")
            continue
        nd = nodes[i]
        k = int(nd["num_parts"])
        if k > 0 or (int(nd["left"]) == 0 and int(nd["right"]) == 0):
            out.append(f"L {k}")
            for j in nd["particles"][:k]:
                p = bodies["p"][int(j)]
                out.append(f"{rust_f64(float(p[0]))} {rust_f64(float(p[1]))} {rust_f64(float(p[2]))}")
        else:
            out.append(f"I {int(nd['split_dim'])} {rust_f64(float(nd['split_val']))} "
                       f"{int(nd['left'])} {int(nd['right'])}")
    return "\n".join(out) + "\n"

"""CPU checks of the Rust FFI crate (rust/kdnbody-sys), which cannot be compiled here (no
cargo in this image): its extern "C" block declares exactly the functions of
include/kdnbody.h with matching parameter and return types, its #[repr(C)] structs have the
header's fields in the header's order and types, and its build script links the library and
the CUDA runtime."""
from __future__ import annotations

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "kdnbody.h"
CRATE = ROOT / "rust" / "kdnbody-sys"
FFI = CRATE / "src" / "ffi.rs"

C_TYPES = {
    "double": "f64", "float": "f32", "size_t": "usize", "int": "c_int", "int32_t": "i32",
    "uint32_t": "u32", "int64_t": "i64", "uint64_t": "u64", "char": "c_char", "void": "c_void",
    "kd_particle_c": "KdParticle", "kd_node_c": "KdNode", "kd_params": "KdParams",
    "kd_stats": "KdStats", "kd_ctx": "KdCtx", "kd_tape": "KdTape",
}


def strip_c_comments(text):
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def c_type_to_rust(decl):
    """'const kd_particle_c *bodies' -> '*const KdParticle'; arrays decay to pointers."""
    decl = decl.strip()
    arr = re.search(r"\[[^\]]*\]$", decl)
    m = re.match(r"(const\s+)?(\w+)\s*((?:\*\s*)*)(\w+)?", decl.replace("[", " [", 1))
    const, base, stars = m.group(1), m.group(2), m.group(3).replace(" ", "")
    n_ptr = len(stars) + (1 if arr else 0)
    t = C_TYPES[base]
    if n_ptr == 0:
        return t
    inner = ("*const " if const else "*mut ") + t
    for _ in range(n_ptr - 1):
        inner = "*mut " + inner
    return inner


def header_functions():
    text = strip_c_comments(HEADER.read_text())
    out = {}
    for m in re.finditer(r"^([A-Za-z_][\w \*]*?)\b(kd_\w+)\s*\(([^)]*)\)\s*;", text, flags=re.M):
        ret = m.group(1).strip()
        args = [a.strip() for a in m.group(3).replace("\n", " ").split(",")]
        args = [] if args == ["void"] or args == [""] else args
        rret = "()" if ret == "void" else c_type_to_rust(ret + " x")
        out[m.group(2)] = (rret, [c_type_to_rust(a) for a in args])
    return out


def rust_functions():
    text = FFI.read_text()
    block = text[text.index('extern "C" {'):]
    out = {}
    for m in re.finditer(r"pub fn (kd_\w+)\(([^)]*)\)\s*(?:->\s*([^;]+))?;", block, flags=re.S):
        args = [a.strip() for a in m.group(2).replace("\n", " ").split(",") if a.strip()]
        types = [re.sub(r"\s+", " ", a.split(":", 1)[1].strip()) for a in args]
        out[m.group(1)] = ((m.group(3) or "()").strip(), types)
    return out


def header_structs():
    text = strip_c_comments(HEADER.read_text())
    out = {}
    for m in re.finditer(r"typedef struct\s*\{([^}]*)\}\s*(\w+)\s*;", text):
        fields = []
        for line in m.group(1).split(";"):
            line = line.strip()
            if not line:
                continue
            fm = re.match(r"(\w+)\s+(\w+)(?:\[(\w+)\])?", line)
            base, name, dim = fm.groups()
            rt = C_TYPES[base]
            if dim:
                rt = f"[{rt}; {'KD_MAX_LEAF' if dim == 'KD_MAX_LEAF' else dim}]"
            fields.append((name, rt))
        out[m.group(2)] = fields
    return out


def rust_structs():
    text = FFI.read_text()
    out = {}
    for m in re.finditer(r"#\[repr\(C\)\][^\n]*\n(?:#\[[^\n]*\n)*pub struct (\w+) \{([^}]*)\}",
                         text):
        fields = re.findall(r"pub (\w+): ([^,]+),", m.group(2))
        out[m.group(1)] = [(n, t.strip()) for n, t in fields]
    return out


def test_extern_block_declares_every_header_function_with_its_types():
    h, r = header_functions(), rust_functions()
    assert set(h) == set(r), (set(h) ^ set(r))
    for name, (ret, args) in h.items():
        rret, rargs = r[name]
        assert rret == ret, (name, rret, ret)
        assert rargs == args, (name, rargs, args)


@pytest.mark.parametrize("c_name,rust_name", [("kd_particle_c", "KdParticle"),
                                              ("kd_node_c", "KdNode"), ("kd_params", "KdParams"),
                                              ("kd_stats", "KdStats")])
def test_repr_c_structs_match_the_header(c_name, rust_name):
    h, r = header_structs(), rust_structs()
    assert r[rust_name] == h[c_name], (r[rust_name], h[c_name])


def test_constants_match_the_header():
    text = strip_c_comments(HEADER.read_text())
    consts = dict(re.findall(r"#define (KD_\w+) \((-?\d+)\)", text))
    consts.update(re.findall(r"#define (KD_\w+) (\d+)", text))
    for name, v in re.findall(r"(KD_\w+) = (-?\d+)", text):
        consts[name] = v
    rs = FFI.read_text()
    for name, v in consts.items():
        m = re.search(rf"pub const {name}: \w+ = (-?\d+);", rs)
        assert m and m.group(1) == v, name


def test_particle_matches_kd_particle_layout():
    """The safe wrapper hands a Vec<Particle> to the library in place."""
    lib = (CRATE / "src" / "lib.rs").read_text()
    m = re.search(r"#\[repr\(C\)\]\s*#\[derive[^\n]*\n\s*pub struct Particle \{([^}]*)\}", lib)
    fields = [(n, t.strip()) for n, t in re.findall(r"pub (\w+): ([^,]+),", m.group(1))]
    assert fields == [("p", "[f64; 3]"), ("v", "[f64; 3]"), ("r", "f64"), ("m", "f64")]


def test_safe_layer_has_the_reference_call_shape():
    lib = (CRATE / "src" / "lib.rs").read_text()
    for sig in [
        "pub fn allocate_node_vec(num_parts: usize) -> Vec<KDTree>",
        "pub fn build_tree(indices: &mut Vec<usize>, start: usize, end: usize,",
        "pub fn build_tree_par4(indices: &mut [usize], cur_node: usize, particles: &Vec<Particle>,",
        "pub fn calc_accel(p: usize, particles: &Vec<Particle>, nodes: &Vec<KDTree>) -> [f64; 3]",
        "pub fn simple_sim(bodies: &mut Vec<Particle>, dt: f64, steps: i64)",
        "pub fn forward(&mut self, dt: f64, steps: i64, ckpt_every: i64) -> Result<Tape<'_>>",
        "pub fn backward(&mut self, dl_dx: &[[f64; 3]], dl_dv: Option<&[[f64; 3]]>)",
        "pub mod array_kd_tree", "pub mod array_particle", "pub mod quickstat",
    ]:
        assert sig in lib, sig


def test_build_script_links_the_library_and_cudart():
    build = (CRATE / "build.rs").read_text()
    assert "cargo:rustc-link-lib=dylib=kdnbody" in build
    assert "cargo:rustc-link-lib=dylib=cudart" in build
    manifest = (CRATE / "Cargo.toml").read_text()
    assert 'links = "kdnbody"' in manifest and 'build = "build.rs"' in manifest

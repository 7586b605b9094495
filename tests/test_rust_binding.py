"""rust/woxel_gb300_ffi.rs (the binding a woxel maintainer adds; no Rust toolchain here to
compile it) against include/woxel_gb300.h: every function of the header is declared
in the binding's extern block with the same parameters in the same order and the
corresponding Rust types; every struct of the header is mirrored field for field; the
status codes have the same values. A change to the header that the binding misses
fails here."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
HEADER = (ROOT / "include" / "woxel_gb300.h").read_text()
RUST = (ROOT / "rust" / "woxel_gb300_ffi.rs").read_text()

C2R = {"int": "c_int", "int32_t": "i32", "uint32_t": "u32", "uint64_t": "u64", "int64_t": "i64", "float": "f32",
       "double": "f64", "uint8_t": "u8", "char": "c_char", "void": "c_void", "size_t": "usize"}


def _strip_comments(s):
    return re.sub(r"//[^\n]*", "", re.sub(r"/\*.*?\*/", "", s, flags=re.S))


def _rust_type(base, const, stars, dims, decay):
    t = C2R.get(base, base)
    if dims and decay:  # an array parameter is a pointer to its first element
        return ("*const " if const else "*mut ") + t
    for k in range(stars):
        t = ("*const " if const and k == 0 else "*mut ") + t
    for n in reversed(dims):
        t = f"[{t}; {n}]"
    return t


def _c_decl(text, decay):
    """(name, Rust type) of one C declaration such as 'const float eye[3]'."""
    m = re.match(r"(const\s+)?([A-Za-z_0-9]+)\s*(\**)\s*(\w+)\s*((?:\[\d+\])*)$", " ".join(text.split()))
    assert m, text
    dims = re.findall(r"\[(\d+)\]", m.group(5))
    return m.group(4), _rust_type(m.group(2), bool(m.group(1)), len(m.group(3)), dims, decay)


def header_functions():
    h = _strip_comments(HEADER)
    out = {}
    for ret, name, params in re.findall(r"^((?:const )?[a-z_0-9]+(?: \*)?)\s*(wx_\w+)\(([^;]*?)\);", h, re.M | re.S):
        ps = [] if params.strip() in ("", "void") else [_c_decl(p, True) for p in params.split(",")]
        r = ret.strip()
        rt = None if r == "void" else _c_decl(r.replace("*", "") + (" *" if "*" in r else "") + " x", False)[1]
        out[name] = (ps, rt)
    return out


def header_structs():
    h = _strip_comments(HEADER)
    out = {}
    for body, name in re.findall(r"typedef struct (?:\w+ )?\{(.*?)\}\s*(wx_\w+);", h, re.S):
        fields = []
        for line in body.split(";"):
            line = " ".join(line.split())
            if not line:
                continue
            m = re.match(r"((?:const )?[A-Za-z_0-9]+)\s*(.*)$", line)
            for d in m.group(2).split(","):
                fields.append(_c_decl(m.group(1) + " " + d.strip(), False))
        out[name] = fields
    return out


def rust_functions():
    block = RUST[RUST.index('extern "C" {'):]
    block = block[: block.index("\n}\n")]
    out = {}
    for name, params, ret in re.findall(r"pub fn (wx_\w+)\((.*?)\)(?:\s*->\s*([^;]+))?;", block, re.S):
        ps = []
        for p in params.split(","):
            p = " ".join(p.split())
            if p:
                n, t = p.split(":", 1)
                ps.append((n.strip(), t.strip()))
        assert name not in out, f"{name} declared twice"
        out[name] = (ps, ret.strip() if ret else None)
    return out


def rust_structs():
    out = {}
    for name, body in re.findall(r"pub struct (wx_\w+) \{(.*?)\n\}", RUST, re.S):
        fields = re.findall(r"pub (\w+): ([^,\n]+),", body)
        out[name] = [(n, " ".join(t.split())) for n, t in fields]
    return out


def test_every_function_is_declared_with_its_signature():
    h, r = header_functions(), rust_functions()
    assert len(h) >= 55
    missing = sorted(set(h) - set(r))
    assert not missing, f"not in the Rust binding: {missing}"
    assert not sorted(set(r) - set(h)), "the Rust binding declares functions the header does not have"
    for name, (ps, rt) in h.items():
        assert r[name][0] == ps, f"{name}: parameters {r[name][0]} != {ps}"
        assert r[name][1] == rt, f"{name}: return type {r[name][1]} != {rt}"


def test_every_struct_is_mirrored():
    h, r = header_structs(), rust_structs()
    for name, fields in h.items():
        if name == "wx_state_uniform":  # the binding uses woxel's own ComputeState (same 256 bytes)
            assert "pub type wx_state_uniform = ComputeState;" in RUST
            continue
        assert name in r, f"struct {name} is not mirrored"
        assert r[name] == fields, f"{name}: {r[name]} != {fields}"
    for opaque in ("wx_ctx", "wx_grid", "wx_topology", "wx_batch", "wx_server"):
        assert re.search(rf"pub struct {opaque} \{{\s*_private: \[u8; 0\],\s*\}}", RUST), opaque


def test_status_codes():
    for name, val in re.findall(r"#define (WX_(?:OK|ERR_\w+)) (\d+)", HEADER):
        assert re.search(rf"pub const {name}: c_int = {val};", RUST), name

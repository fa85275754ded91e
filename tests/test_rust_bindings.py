"""The Rust binding source (rust/ndarray-conv-sys) stays in step with the C
header: every function include/ndconv.h declares has an extern "C"
declaration of the same name and number of arguments, nothing else is
declared, and the #[repr(C)] ndconv_problem has the C struct's fields in the
same order with the same element types and array lengths.  No Rust toolchain
is involved: both files are read as text.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ndconv.h")
SYS = os.path.join(ROOT, "rust", "ndarray-conv-sys", "src", "lib.rs")


def _strip_c_comments(s):
    return re.sub(r"/\*.*?\*/", "", s, flags=re.S)


def _arity(args):
    args = " ".join(args.split())
    if args in ("", "void"):
        return 0
    return len([a for a in args.split(",") if a.strip()])


def c_functions():
    s = _strip_c_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"^\s*(?:const\s+)?\w+\s*\*?\s*(ndconv_\w+)\s*\(([^;]*?)\)\s*;", s, re.M):
        out[m.group(1)] = _arity(m.group(2))
    return out


def rust_functions():
    s = open(SYS).read()
    block = s[s.index('#[link(name = "ndconv")]'):]
    block = block[:block.index("\n}\n")]
    block = re.sub(r"//[^\n]*", "", block)
    out = {}
    for m in re.finditer(r"pub fn (ndconv_\w+)\s*\((.*?)\)\s*(?:->\s*[^;]+)?;", block, re.S):
        out[m.group(1)] = _arity(m.group(2))
    return out


def test_every_header_function_is_bound_with_its_arity():
    c, r = c_functions(), rust_functions()
    assert len(c) >= 30
    assert sorted(c) == sorted(r), (sorted(set(c) - set(r)), sorted(set(r) - set(c)))
    for name, n in c.items():
        assert r[name] == n, (name, n, r[name])


C_TO_RUST = {"int32_t": "i32", "int64_t": "i64", "double": "f64"}


def test_problem_struct_layout_matches():
    s = _strip_c_comments(open(HEADER).read())
    body = re.search(r"typedef struct ndconv_problem \{(.*?)\} ndconv_problem;", s, re.S).group(1)
    cfields = []
    for m in re.finditer(r"(\w+)\s+(\w+)((?:\[\d+\])*)\s*;", body):
        dims = [int(d) for d in re.findall(r"\[(\d+)\]", m.group(3))]
        cfields.append((m.group(2), C_TO_RUST[m.group(1)], dims))
    rs = open(SYS).read()
    rbody = re.search(r"pub struct ndconv_problem \{(.*?)\n\}", rs, re.S).group(1)
    rfields = []
    for m in re.finditer(r"pub (\w+):\s*([^,\n]+),", rbody):
        t = m.group(2).strip()
        dims = []
        while t.startswith("["):
            inner, n = re.fullmatch(r"\[(.*);\s*(\d+)\]", t).groups()
            dims.append(int(n))
            t = inner.strip()
        rfields.append((m.group(1), t, dims))
    assert cfields == rfields


def test_safe_crate_exports_the_reference_api():
    lib = open(os.path.join(ROOT, "rust", "ndarray-conv", "src", "lib.rs")).read()
    for name in ("ConvExt", "ConvFFTExt", "get_fft_processor", "GetProcessor", "FftProcessor", "ReverseKernel",
                 "WithDilation", "enum ConvMode", "enum PaddingMode", "enum BorderType", "enum Error"):
        assert name in lib, name

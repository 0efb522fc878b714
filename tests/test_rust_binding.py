"""The Rust binding (rust/omg-cuda/src/lib.rs) against the C header, as text:
there is no Rust toolchain here, so its #[repr(C)] structs are checked field
by field (names, element types and counts, order) against the header's
structs, and every function of its extern block against the header's
declarations (name and argument count), together with the ABI version."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "omg_cuda.h")
RUST = os.path.join(ROOT, "rust", "omg-cuda", "src", "lib.rs")

C_TYPES = {"uint32_t": "u32", "int32_t": "i32", "float": "f32", "uint64_t": "u64"}
PAIRS = {"OmgMaterial": "omg_material", "OmgParams": "omg_params", "OmgBoxJob": "omg_box_job",
         "OmgWorldJob": "omg_world_job", "OmgPanel": "omg_panel", "OmgReverb": "omg_reverb"}


def _strip_c_comments(s):
    return re.sub(r"/\*.*?\*/", "", s, flags=re.S)


def _c_structs():
    text = _strip_c_comments(open(HEADER).read())
    defines = {k: int(v) for k, v in re.findall(r"#define (\w+) \(?(\d+)u?\)?\s", text)}
    out = {}
    for body, name in re.findall(r"typedef struct \w+ \{(.*?)\} (\w+);", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.fullmatch(r"(\w+) (.+)", decl)
            ctype, names = m.group(1), m.group(2)
            for nm in names.split(","):
                nm = nm.strip()
                a = re.fullmatch(r"(\w+)(?:\[(\w+)\])?", nm)
                count = a.group(2)
                count = (defines[count] if count in defines else int(count)) if count else 1
                fields.append((a.group(1), C_TYPES.get(ctype, ctype), count))
        out[name] = fields
    return out


def _rust_structs():
    text = open(RUST).read()
    out = {}
    for name, body in re.findall(r"#\[repr\(C\)\]\s*(?:#\[[^\]]*\]\s*)*(?:pub )?struct (\w+) \{(.*?)\}", text,
                                 flags=re.S):
        fields = []
        for line in body.split(","):
            line = line.strip()
            if not line:
                continue
            m = re.fullmatch(r"(?:pub )?(\w+): (.+)", line)
            ty = m.group(2).strip()
            a = re.fullmatch(r"\[(\w+); (\w+)\]", ty)
            if a:
                count = 8 if a.group(2) == "MAXB" else int(a.group(2))
                ty = a.group(1)
            else:
                count = 1
            fields.append((m.group(1), PAIRS.get(ty, ty), count))
        out[name] = fields
    return out


def test_repr_c_structs_match_the_header():
    c, r = _c_structs(), _rust_structs()
    assert set(PAIRS) <= set(r), sorted(r)
    for rust_name, c_name in PAIRS.items():
        assert r[rust_name] == c[c_name], (rust_name, r[rust_name], c[c_name])


def test_extern_functions_are_declared_in_the_header():
    header = _strip_c_comments(open(HEADER).read())
    text = open(RUST).read()
    block = re.search(r'extern "C" \{(.*?)\n\}', text, flags=re.S).group(1)
    fns = re.findall(r"fn (\w+)\((.*?)\)", block, flags=re.S)
    assert len(fns) >= 10
    for name, args in fns:
        m = re.search(r"\b" + name + r"\s*\((.*?)\)\s*;", header, flags=re.S)
        assert m, name
        n_c = 0 if m.group(1).strip() in ("", "void") else m.group(1).count(",") + 1
        n_r = 0 if not args.strip() else args.count(",") + 1
        assert n_c == n_r, (name, n_c, n_r)


def test_abi_version_matches():
    v_c = int(re.search(r"#define OMG_ABI_VERSION (\d+)", open(HEADER).read()).group(1))
    v_r = int(re.search(r"pub const ABI_VERSION: i32 = (\d+);", open(RUST).read()).group(1))
    assert v_c == v_r

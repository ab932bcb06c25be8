"""The C-ABI library: builds, loads, exports what include/puck_gpu.h declares,
and reads grammar artifacts on the host (no GPU calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

from puck_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def declared_functions():
    src = open(os.path.join(ROOT, "include", "puck_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(puck_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    assert set(names) >= set(_lib.EXPORTS)


def test_options_layout_and_defaults():
    """The ctypes mirror of puck_options has the C layout (48 bytes:
    server_lanes at 40, then padding to the int64 alignment) and the
    library's defaults."""
    L = _lib.load()
    assert ctypes.sizeof(_lib.Options) == 48
    assert _lib.Options.tensor_cores.offset == 36
    assert _lib.Options.server_lanes.offset == 40
    opt = _lib.Options()
    opt.tensor_cores = 7
    opt.server_lanes = 5
    L.puck_default_options(ctypes.byref(opt))
    assert opt.tensor_cores == 0 and opt.use_graphs == 0 and abs(opt.prune_threshold + 9.0) < 1e-6
    assert opt.server_lanes == 0


def test_tc_selftest_rejects_bad_shapes_without_a_device_call():
    L = _lib.load()
    z = np.zeros(128 * 32, np.uint16)
    d = np.zeros(128 * 32, np.float32)
    for k, n in ((24, 16), (16, 8), (0, 16), (272, 16), (16, 272)):
        assert L.puck_tc_selftest(0, k, n, z.ctypes.data, z.ctypes.data, d.ctypes.data) == 6


def test_grammar_load_and_queries_on_host():
    L = _lib.load()
    st = ctypes.c_int32(-1)
    g = L.puck_grammar_load(os.path.join(GOLDEN, "split_cascade_viterbi.grz").encode(), ctypes.byref(st))
    assert g and st.value == 0
    try:
        assert L.puck_grammar_num_levels(g) == 2
        info = (ctypes.c_int32 * 8)()
        assert L.puck_grammar_level_info(g, 1, info) == 0
        semiring, n_nt, n_t, cs, ms, nc, root, nw = list(info)
        assert semiring == 0 and cs % 32 == 0 and cs >= max(n_nt, n_t) and nw == 300
        assert L.puck_grammar_word_id(g, b"w17") == 17
        assert L.puck_grammar_word_id(g, b"no-such-word") == -1
        assert L.puck_grammar_level_info(g, 5, info) == 6
    finally:
        L.puck_grammar_free(g)


def test_bad_artifacts_fail_cleanly(tmp_path):
    L = _lib.load()
    st = ctypes.c_int32(0)
    assert not L.puck_grammar_load(str(tmp_path / "missing.grz").encode(), ctypes.byref(st))
    assert st.value == 2 and "cannot open" in _lib.last_error()
    p = tmp_path / "trunc.grz"
    data = open(os.path.join(GOLDEN, "tiny_pcfg_viterbi.grz"), "rb").read()
    p.write_bytes(data[: len(data) // 2])
    assert not L.puck_grammar_load(str(p).encode(), ctypes.byref(st))
    assert st.value == 2
    import zipfile
    q = tmp_path / "deflated.grz"
    with zipfile.ZipFile(q, "w", compression=zipfile.ZIP_DEFLATED) as z:
        z.writestr("parserNames", "parser-0")
        z.writestr("parser-0/header", "semiring viterbi\n")
    assert not L.puck_grammar_load(str(q).encode(), ctypes.byref(st))
    assert st.value == 2


def _patched(tmp_path, name, patch):
    """A copy of a valid archive with ``patch(bytearray, eocd, cd)`` applied."""
    import struct
    data = bytearray(open(os.path.join(GOLDEN, "tiny_pcfg_viterbi.grz"), "rb").read())
    eocd = data.rindex(b"PK\x05\x06")
    cd = struct.unpack_from("<I", data, eocd + 16)[0]
    patch(data, eocd, cd)
    p = tmp_path / name
    p.write_bytes(bytes(data))
    return str(p).encode()


def test_corrupt_offsets_and_counts_fail_cleanly(tmp_path):
    """Fields read from the file are bounded before use: an entry name
    running past the end, a local-header offset near 2^32, an array element
    count that is negative or overflows its byte size."""
    import struct
    L = _lib.load()
    st = ctypes.c_int32(0)

    def last_entry_long_name(d, eocd, cd):
        n = struct.unpack_from("<H", d, eocd + 10)[0]
        for _ in range(n - 1):                      # walk to the last central-directory entry
            nl, xl, cl = struct.unpack_from("<HHH", d, cd + 28)
            cd += 46 + nl + xl + cl
        struct.pack_into("<H", d, cd + 28, 0xFFFF)

    def huge_local_offset(d, eocd, cd):
        struct.pack_into("<I", d, cd + 42, 0xFFFFFFF0)

    for name, patch, msg in (("name.grz", last_entry_long_name, "corrupt central directory"),
                             ("lho.grz", huge_local_offset, "corrupt local header")):
        assert not L.puck_grammar_load(_patched(tmp_path, name, patch), ctypes.byref(st))
        assert st.value == 2 and msg in _lib.last_error(), _lib.last_error()

    import zipfile
    src = os.path.join(GOLDEN, "tiny_pcfg_viterbi.grz")
    for count in (-1, -(1 << 62), 1 << 62, (1 << 63) - 1):
        q = tmp_path / f"count{count & 0xff}.grz"
        with zipfile.ZipFile(src) as zin, zipfile.ZipFile(q, "w", zipfile.ZIP_STORED) as zout:
            for info in zin.infolist():
                data = zin.read(info.filename)
                if info.filename == "parser-0/arrays/in_NN/w":
                    data = data[:8] + struct.pack("<q", count) + data[16:]
                zout.writestr(zipfile.ZipInfo(info.filename, date_time=(1980, 1, 1, 0, 0, 0)), data)
        assert not L.puck_grammar_load(str(q).encode(), ctypes.byref(st))
        assert st.value == 2 and "truncated parser-0/arrays/in_NN/w" in _lib.last_error(), _lib.last_error()


def test_build_flags_target_sm103a():
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def _compile_via_abi(prefixes, out, viterbi=1, logsum=0):
    L = _lib.load()
    L.puck_compile_grammar.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_void_p]
    L.puck_compile_grammar.restype = ctypes.c_int32
    opts = (ctypes.c_int32 * 4)()
    L.puck_default_compile_options(ctypes.byref(opts))
    opts[0], opts[1] = viterbi, logsum
    return L.puck_compile_grammar(prefixes.encode(), out.encode(), ctypes.byref(opts))


def _same_archives(a, b):
    import zipfile
    za, zb = zipfile.ZipFile(a), zipfile.ZipFile(b)
    names = sorted(za.namelist())
    assert names == sorted(zb.namelist())
    for n in names:
        assert za.read(n) == zb.read(n), n


def test_compile_grammar_through_the_c_abi_matches_the_python_compiler(tmp_path):
    """puck_compile_grammar (CompileGrammar behind the C ABI) writes the same
    archive, entry for entry, as the compile_grammar program, for a Viterbi
    and a LogSum fine level, and reports unreadable input as BAD_GRAMMAR."""
    from helpers import write_text_grammar
    from puck_gb300 import compile_grammar
    c = write_text_grammar(str(tmp_path), "coarse", 1, seed=1)
    f = write_text_grammar(str(tmp_path), "fine", 2, seed=2)
    for vit, ls, sem in ((1, 0, "viterbi"), (0, 1, "logsum")):
        abi, py = str(tmp_path / f"abi_{sem}.grz"), str(tmp_path / f"py_{sem}.grz")
        assert _compile_via_abi(f"{c}:{f}", abi, vit, ls) == 0, _lib.last_error()
        assert compile_grammar.main(["--textGrammarPrefix", f"{c}:{f}", "--grammar", py,
                                     "--viterbi", str(bool(vit)).lower(), "--logsum", str(bool(ls)).lower()]) == 0
        _same_archives(abi, py)
    assert _compile_via_abi(str(tmp_path / "missing"), str(tmp_path / "x.grz")) == 2
    assert "missing" in _lib.last_error()
    L = _lib.load()
    opts = (ctypes.c_int32 * 4)()
    L.puck_default_compile_options(ctypes.byref(opts))
    # reproject through the C ABI equals the command line's --reproject
    from test_cli import _hierarchy_pair
    hc, hf = _hierarchy_pair(tmp_path)
    opts[2] = 1  # reproject
    abi, py = str(tmp_path / "r_abi.grz"), str(tmp_path / "r_py.grz")
    assert L.puck_compile_grammar(f"{hc}:{hf}".encode(), abi.encode(), ctypes.byref(opts)) == 0, _lib.last_error()
    assert compile_grammar.main(["--textGrammarPrefix", f"{hc}:{hf}", "--grammar", py, "--reproject"]) == 0
    _same_archives(abi, py)


def test_compile_grammar_from_a_host_without_python(tmp_path):
    """A C host that loads only libpuck_gb300.so (no Python in the process,
    like a JVM): puck_compile_grammar starts its own interpreter and writes
    the same archive."""
    import shutil
    import subprocess
    from helpers import write_text_grammar
    from puck_gb300 import compile_grammar
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    c = write_text_grammar(str(tmp_path), "coarse", 1, seed=3)
    f = write_text_grammar(str(tmp_path), "fine", 3, seed=4)
    src = tmp_path / "host.c"
    src.write_text(
        '#include <dlfcn.h>\n#include <stdio.h>\n#include "puck_gpu.h"\n'
        "int main(int argc, char** argv) {\n"
        "  void* h = dlopen(argv[1], RTLD_NOW);\n"
        "  if (!h) { fprintf(stderr, \"%s\\n\", dlerror()); return 3; }\n"
        "  puck_status (*compile)(const char*, const char*, const puck_compile_options*) =\n"
        "      (puck_status (*)(const char*, const char*, const puck_compile_options*))dlsym(h, \"puck_compile_grammar\");\n"
        "  size_t (*err)(char*, size_t) = (size_t (*)(char*, size_t))dlsym(h, \"puck_last_error\");\n"
        "  puck_status st = compile(argv[2], argv[3], NULL);\n"
        "  char msg[512]; msg[0] = 0; if (st) err(msg, sizeof msg);\n"
        "  printf(\"%d %s\\n\", (int)st, msg);\n"
        "  return st == PUCK_OK ? 0 : 1;\n}\n")
    exe = tmp_path / "host"
    subprocess.check_call(["gcc", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-ldl"])
    out = str(tmp_path / "c_host.grz")
    r = subprocess.run([str(exe), build.build(), f"{c}:{f}", out], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    py = str(tmp_path / "py.grz")
    assert compile_grammar.main(["--textGrammarPrefix", f"{c}:{f}", "--grammar", py]) == 0
    _same_archives(out, py)


def _c_kind(ctype: str) -> str:
    t = ctype.strip()
    if "*" in t or "[" in t:
        return "ADDRESS"
    base = t.replace("const", "").split()[-1]
    return {"int64_t": "JAVA_LONG", "size_t": "JAVA_LONG", "int32_t": "JAVA_INT", "puck_status": "JAVA_INT",
            "int": "JAVA_INT", "float": "JAVA_FLOAT", "double": "JAVA_DOUBLE"}[base]


def test_panama_binding_in_integration_doc_matches_header():
    """The JVM binding shown for maintainers cannot be compiled here (no
    JDK); its downcall descriptors are checked against the C declarations
    instead: every bound name exists, with the same argument count, argument
    and return kinds, and puck_options' layout has the header's fields in
    order and its 48 bytes."""
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    hdr = open(os.path.join(root, "include", "puck_gpu.h")).read()
    hdr = re.sub(r"/\*.*?\*/", " ", hdr, flags=re.S)
    protos = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(puck_\w+)\s*\(([^)]*)\)\s*;", hdr):
        ret, name, args = m.group(1).split(";")[-1].split("}")[-1].strip(), m.group(2), m.group(3).strip()
        params = [] if args in ("", "void") else [a.rsplit(None, 1)[0] if not a.strip().endswith("]")
                                                  else a for a in args.split(",")]
        protos[name] = (None if ret == "void" else _c_kind(ret), [_c_kind(p) for p in params])
    doc = open(os.path.join(root, "INTEGRATION.md")).read()
    java = doc[doc.index("```java"):]
    java = java[:java.index("```", 7)]
    bound = re.findall(r'h\("(puck_\w+)",\s*FunctionDescriptor\.(ofVoid|of)\(([^)]*)\)\)', java, flags=re.S)
    assert len(bound) >= 8
    for name, form, items in bound:
        kinds = [k.strip() for k in items.split(",") if k.strip()]
        ret = None if form == "ofVoid" else kinds.pop(0)
        assert name in protos, name
        assert (ret, kinds) == protos[name], (name, (ret, kinds), protos[name])
    fields = re.search(r"typedef struct puck_options \{(.*?)\} puck_options;", hdr, flags=re.S).group(1)
    c_fields = [(_c_kind(f.rsplit(None, 1)[0]), f.rsplit(None, 1)[1]) for f in
                (x.strip() for x in fields.split(";")) if f]
    layout = re.search(r"structLayout\((.*?)\);", java, flags=re.S).group(1)
    j_fields = re.findall(r"(JAVA_\w+)\.withName\(\"(\w+)\"\)", layout)
    assert j_fields == c_fields
    size = {"JAVA_LONG": 8, "JAVA_INT": 4, "JAVA_FLOAT": 4}
    pad = sum(int(x) for x in re.findall(r"paddingLayout\((\d+)\)", layout))
    assert sum(size[k] for k, _ in j_fields) + pad == 48


def test_ctypes_binding_matches_header():
    """Every entry point the Python side binds has the header's argument
    count and kinds (pointer, 32-bit, 64-bit, float) and return kind."""
    import ctypes
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    hdr = re.sub(r"/\*.*?\*/", " ", open(os.path.join(root, "include", "puck_gpu.h")).read(), flags=re.S)
    protos = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(puck_\w+)\s*\(([^)]*)\)\s*;", hdr):
        ret, name, args = m.group(1).split(";")[-1].split("}")[-1].strip(), m.group(2), m.group(3).strip()
        params = [] if args in ("", "void") else [a if a.strip().endswith("]") else a.rsplit(None, 1)[0]
                                                  for a in args.split(",")]
        protos[name] = (None if ret == "void" else _c_kind(ret), [_c_kind(p) for p in params])

    def kind(t):
        if t is None:
            return None
        if t in (ctypes.c_void_p, ctypes.c_char_p) or issubclass(t, ctypes._Pointer):
            return "ADDRESS"
        return {ctypes.c_int32: "JAVA_INT", ctypes.c_int64: "JAVA_LONG", ctypes.c_size_t: "JAVA_LONG",
                ctypes.c_float: "JAVA_FLOAT", ctypes.c_double: "JAVA_DOUBLE"}[t]

    L = _lib.load()
    assert set(_lib.EXPORTS) == set(protos)
    for name in _lib.EXPORTS:
        f = getattr(L, name)
        assert f.argtypes is not None, name
        want_ret, want_args = protos[name]
        got_ret = None if f.restype is None else kind(f.restype)
        if want_ret is None:
            # ctypes' default restype is c_int; a void function may keep it
            assert got_ret in (None, "JAVA_INT"), name
        else:
            assert got_ret == want_ret, (name, got_ret, want_ret)
        assert [kind(t) for t in f.argtypes] == want_args, (name, [kind(t) for t in f.argtypes], want_args)


def test_python_mirror_keeps_the_reference_names():
    """CLParser / CLParserData carry the reference's method names beside the
    Python ones (parse, partitions, insideOutside, release, isViterbi,
    readSequence, writeSequence)."""
    from puck_gb300.parser import CLParser, CLParserData
    for name in ("parse", "partitions", "insideOutside", "release", "isViterbi"):
        assert hasattr(CLParser, name), name
    assert CLParser.insideOutside is CLParser.inside_outside
    assert CLParser.isViterbi is CLParser.is_viterbi
    for name in ("readSequence", "writeSequence", "isViterbi"):
        assert hasattr(CLParserData, name), name
    from helpers import small_pcfg_levels, write_grz
    data = CLParserData.readSequence(write_grz(small_pcfg_levels(), "names_check"))
    assert len(data) == 1 and data[0].isViterbi and data[0].is_viterbi


def _with_array(tmp_path, name, entry, fn):
    """A copy of a valid archive whose array ``entry`` (of level 0) has its
    elements passed through ``fn(numpy array) -> numpy array``."""
    import zipfile
    import numpy as np
    src = os.path.join(GOLDEN, "tiny_pcfg_viterbi.grz")
    q = tmp_path / name
    with zipfile.ZipFile(src) as zin, zipfile.ZipFile(q, "w", zipfile.ZIP_STORED) as zout:
        for info in zin.infolist():
            data = zin.read(info.filename)
            if info.filename == f"parser-0/arrays/{entry}":
                tag = data[4:8].rstrip(b"\0 ").decode()
                dt = {"i4": np.int32, "i8": np.int64, "f4": np.float32}[tag[:2]]
                vals = fn(np.frombuffer(data[16:], dt).copy()).astype(dt)
                data = data[:16] + vals.tobytes()
            zout.writestr(zipfile.ZipInfo(info.filename, date_time=(1980, 1, 1, 0, 0, 0)), data)
    return str(q).encode()


def test_tables_the_device_walks_are_validated_at_load(tmp_path):
    """Offset tables that are not 0-based and non-decreasing, backtrace
    symbols out of range and NaN weights are refused when the archive is
    loaded, before any device table is built from them."""
    import numpy as np
    L = _lib.load()
    st = ctypes.c_int32(0)

    def swap_middle(v):
        k = len(v) // 2
        v[k], v[k + 1] = v[k + 1] + 1, v[k]   # a step down inside the table
        return v

    def first(x):
        def f(v):
            v[0] = x
            return v
        return f

    cases = [
        ("lex_off", swap_middle, "bad offsets in lex_off"),
        ("v_off", swap_middle, "bad offsets in v_off"),
        ("nt_mem_off", first(1), "bad offsets in nt_mem_off"),
        ("in_NU/rowptr", swap_middle, "bad offsets in in_NU/rowptr"),
        ("in_NN/pair_blk", swap_middle, "bad offsets in in_NN/pair_blk"),
        ("in_NN/blk_ptr", swap_middle, "bad offsets in in_NN/blk_ptr"),
        ("v_left", first(1 << 20), "index out of range in v_left"),
        ("v_right", first(-1), "index out of range in v_right"),
        ("in_NN/w", first(np.nan), "NaN weight in in_NN/w"),
        ("lex_score", first(np.nan), "NaN weight in lex_score"),
    ]
    for entry, fn, msg in cases:
        p = _with_array(tmp_path, entry.replace("/", "_") + ".grz", entry, fn)
        assert not L.puck_grammar_load(p, ctypes.byref(st)), entry
        assert st.value == 2 and msg in _lib.last_error(), (entry, _lib.last_error())
    # a header whose mask words cannot hold every coarse symbol
    import zipfile
    q = tmp_path / "mask.grz"
    with zipfile.ZipFile(os.path.join(GOLDEN, "tiny_pcfg_viterbi.grz")) as zin, \
            zipfile.ZipFile(q, "w", zipfile.ZIP_STORED) as zout:
        for info in zin.infolist():
            data = zin.read(info.filename)
            if info.filename == "parser-0/header":
                lines = [l for l in data.decode().splitlines() if l]
                data = "".join((f"n_coarse 40\n" if l.startswith("n_coarse ") else l + "\n")
                               for l in lines).encode()
            zout.writestr(zipfile.ZipInfo(info.filename, date_time=(1980, 1, 1, 0, 0, 0)), data)
    assert not L.puck_grammar_load(str(q).encode(), ctypes.byref(st))
    assert st.value == 2 and "mask size does not cover" in _lib.last_error(), _lib.last_error()
    # -inf stays a legal log weight
    p = _with_array(tmp_path, "neginf.grz", "in_NN/w", first(-np.inf))
    g = L.puck_grammar_load(p, ctypes.byref(st))
    assert g and st.value == 0
    L.puck_grammar_free(g)


def test_randomly_corrupted_archives_load_or_fail_cleanly(tmp_path):
    """Seeded corruption of a valid archive (truncation, bit flips, byte
    noise, zeroed runs): every load either succeeds or returns
    PUCK_ERR_BAD_GRAMMAR with a message; none crashes."""
    import random
    L = _lib.load()
    st = ctypes.c_int32(0)
    src = open(os.path.join(GOLDEN, "split_cascade_viterbi.grz"), "rb").read()
    rng = random.Random(2026)
    outcomes = {0: 0, 2: 0}
    for it in range(150):
        b = bytearray(src)
        kind = it % 4
        if kind == 0:
            b = b[:rng.randrange(len(b))]
        elif kind == 1:
            for _ in range(rng.randint(1, 4)):
                b[rng.randrange(len(b))] ^= 1 << rng.randrange(8)
        elif kind == 2:
            for _ in range(rng.randint(20, 200)):
                b[rng.randrange(len(b))] = rng.randrange(256)
        else:
            s = rng.randrange(len(b))
            n = min(rng.randint(4, 4096), len(b) - s)
            b[s:s + n] = bytes(n)
        p = tmp_path / f"c{it}.grz"
        p.write_bytes(bytes(b))
        g = L.puck_grammar_load(str(p).encode(), ctypes.byref(st))
        assert st.value in (0, 2), (it, st.value)
        assert bool(g) == (st.value == 0)
        if g:
            out = (ctypes.c_int32 * 8)()
            for lv in range(L.puck_grammar_num_levels(g)):
                assert L.puck_grammar_level_info(g, lv, out) == 0
            L.puck_grammar_free(g)
        else:
            assert _lib.last_error()
        outcomes[st.value] += 1
    assert outcomes[2] > 100

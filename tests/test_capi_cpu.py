"""Host-side checks of libculsh that need no GPU: the library loads and exports
every entry point of include/culsh.h, the index file layout round-trips
byte for byte, corrupt files and bad arguments fail with the right status,
compute without a GPU fails loudly, and the drop-in C++ header compiles and
links."""

import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, cuda_device_count, load_case

HEADER = os.path.join(ROOT, "include", "culsh.h")
INDEX_BIN = os.path.join(GOLDEN, "odd_d13.index.bin")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(culsh_[A-Za-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(culsh):
    names = declared_functions()
    assert len(names) >= 30
    lib = culsh.lib()
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(culsh.ABI) == names, "python bindings must cover the header exactly"
    assert culsh.lib().culsh_version() >= 10000


def test_nm_lists_the_exports(culsh):
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", "--defined-only", culsh.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (culsh_[A-Za-z_0-9]+)", out))
    assert set(declared_functions()) <= exported


def test_load_getters_and_byte_identical_save(culsh, tmp_path):
    c = load_case("odd_d13")
    ht = culsh.HashTables()
    ht.load(INDEX_BIN)
    L, M, D = c["A"].shape
    assert (ht.getN(), ht.getD(), ht.getL(), ht.getM()) == (c["X"].shape[0], D, L, M)
    assert ht.getW() == float(c["W"])
    np.testing.assert_array_equal(ht.getBuckets(), c["buckets"])
    for l in range(L):
        np.testing.assert_array_equal(ht.getA(l), c["A"][l])
        np.testing.assert_array_equal(ht.getb(l), c["b"][l])
        assert ht.getBuckets(l) == c["buckets"][l]
        np.testing.assert_array_equal(ht.getBuckets_totalIndices(l), c[f"ids_{l}"])
        np.testing.assert_array_equal(ht.getBuckets_startingIndices(l), c[f"starts_{l}"])
        np.testing.assert_array_equal(ht.getBuckets_sizes(l), c[f"sizes_{l}"])
        np.testing.assert_array_equal(ht.getBuckets_codes(l), c[f"codes_{l}"])
    out = tmp_path / "again.bin"
    ht.save(str(out))
    assert out.read_bytes() == open(INDEX_BIN, "rb").read()
    ht2 = culsh.HashTables()
    ht2.reset(str(out))   # reset(filename) is load()
    np.testing.assert_array_equal(ht2.getBuckets_codes(1), c["codes_1"])


def _expect(culsh, code, fn, *a, **k):
    with pytest.raises(culsh.CulshError) as ei:
        fn(*a, **k)
    assert ei.value.code == code, str(ei.value)
    return str(ei.value)


def test_corrupt_index_files_are_rejected(culsh, tmp_path):
    raw = open(INDEX_BIN, "rb").read()
    ht = culsh.HashTables()
    _expect(culsh, culsh.ERR_IO, ht.load, str(tmp_path / "missing.bin"))
    p = tmp_path / "t.bin"
    p.write_bytes(raw[:10])
    _expect(culsh, culsh.ERR_FORMAT, ht.load, str(p))
    p.write_bytes(raw[:-4])
    _expect(culsh, culsh.ERR_FORMAT, ht.load, str(p))
    p.write_bytes(raw + b"\0\0\0\0")
    _expect(culsh, culsh.ERR_FORMAT, ht.load, str(p))
    bad = bytearray(raw)
    bad[12:16] = np.int32(0).tobytes()      # M = 0
    p.write_bytes(bytes(bad))
    _expect(culsh, culsh.ERR_FORMAT, ht.load, str(p))
    # Break the first bucket start of table 0 (must be 0).
    c = load_case("odd_d13")
    N = c["X"].shape[0]
    L, M, D = c["A"].shape
    off = 20 + 4 * L * (D * M + M) + 4 * L + 4 * N
    bad = bytearray(raw)
    bad[off:off + 4] = np.uint32(5).tobytes()
    p.write_bytes(bytes(bad))
    _expect(culsh, culsh.ERR_FORMAT, ht.load, str(p))
    # An id out of range.
    bad = bytearray(raw)
    bad[20 + 4 * L * (D * M + M) + 4 * L: 24 + 4 * L * (D * M + M) + 4 * L] = np.uint32(N + 7).tobytes()
    p.write_bytes(bytes(bad))
    _expect(culsh, culsh.ERR_FORMAT, ht.load, str(p))
    # A valid load still works afterwards.
    ht.load(INDEX_BIN)
    assert ht.getL() == L


def test_parameter_and_state_errors(culsh):
    ht = culsh.HashTables()
    A = np.zeros((1, 2, 3), np.float32)
    b = np.zeros((1, 2), np.float32)
    _expect(culsh, culsh.ERR_INVALID_ARGUMENT, ht.reset, 10, 3, 1, 0, 1.0, A=A[:, :0], b=b[:, :0])
    _expect(culsh, culsh.ERR_INVALID_ARGUMENT, ht.reset, 10, 3, 1, 2, -1.0, A=A, b=b)
    _expect(culsh, culsh.ERR_INVALID_ARGUMENT, ht.reset, 0, 3, 1, 2, 1.0, A=A, b=b)
    big = np.zeros((1, 65, 3), np.float32)
    _expect(culsh, culsh.ERR_CAPACITY, ht.reset, 10, 3, 1, 65, 1.0, A=big, b=np.zeros((1, 65), np.float32))
    _expect(culsh, culsh.ERR_CAPACITY, ht.reset, 1 << 30, 3, 1, 2, 1.0, A=A, b=b)
    fresh = culsh.HashTables()
    _expect(culsh, culsh.ERR_STATE, fresh.index, np.zeros(0, np.float32))
    _expect(culsh, culsh.ERR_STATE, fresh.save, "/nonexistent/x.bin")
    st = culsh.SearchTables()
    _expect(culsh, culsh.ERR_STATE, st.search_device, 0, 1, 0, 0)  # no index attached
    ht.reset(10, 3, 1, 2, 1.0, A=A, b=b)
    st.reset(ht, 5, 1)
    _expect(culsh, culsh.ERR_STATE, st.search, np.zeros((1, 3), np.float32), 1, None)  # not indexed
    loaded = culsh.HashTables()
    loaded.load(INDEX_BIN)
    st.reset(loaded, 0, 1)
    _expect(culsh, culsh.ERR_INVALID_ARGUMENT, st.search, np.zeros((1, 13), np.float32), 1, None)
    st.reset(loaded, culsh.MAX_K + 1, 1)
    _expect(culsh, culsh.ERR_CAPACITY, st.search, np.zeros((1, 13), np.float32), 1, None)
    st.reset(loaded, 5, culsh.MAX_T + 1)
    _expect(culsh, culsh.ERR_CAPACITY, st.search, np.zeros((1, 13), np.float32), 1, None)


@pytest.mark.skipif(cuda_device_count() > 0, reason="checks the no-GPU behaviour")
def test_compute_without_gpu_fails_loudly(culsh):
    c = load_case("odd_d13")
    ht = culsh.HashTables()
    ht.load(INDEX_BIN)
    st = culsh.SearchTables()
    st.reset(ht, 5, 2)
    msg = _expect(culsh, culsh.ERR_CUDA, st.search, c["queries"], None, c["X"])
    assert "device" in msg.lower() or "cuda" in msg.lower()
    assert st.getKnnIds() is None
    L, M, D = c["A"].shape
    ht2 = culsh.HashTables()
    ht2.reset(c["X"].shape[0], D, L, M, float(c["W"]), A=c["A"], b=c["b"])
    _expect(culsh, culsh.ERR_CUDA, ht2.index, c["X"])


DROPIN_SRC = r"""
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include "cuLSH.h"
// Reads: N D L M W Q K T, then A (L*D*M), b (L*M), X (N*D), queries (Q*D) as raw float32
// from argv[1]; writes ids (Q*K int32), dists (Q*K f32), per-table query buckets,
// and the index file to argv[2], argv[2].index.
int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = fopen(argv[1], "rb");
    int hdr[8]; float W;
    if (fread(hdr, 4, 5, f) != 5) return 3;
    W = *reinterpret_cast<float*>(&hdr[4]);
    if (fread(&hdr[5], 4, 3, f) != 3) return 3;
    const int N = hdr[0], D = hdr[1], L = hdr[2], M = hdr[3], Q = hdr[5], K = hdr[6], T = hdr[7];
    std::vector<std::vector<float>> A(L, std::vector<float>(D * M)), b(L, std::vector<float>(M));
    std::vector<float*> Ap(L), bp(L);
    for (int l = 0; l < L; ++l) { if (fread(A[l].data(), 4, D * M, f) != (size_t)(D * M)) return 3; Ap[l] = A[l].data(); }
    for (int l = 0; l < L; ++l) { if (fread(b[l].data(), 4, M, f) != (size_t)M) return 3; bp[l] = b[l].data(); }
    std::vector<float> X((size_t)N * D), q((size_t)Q * D);
    if (fread(X.data(), 4, X.size(), f) != X.size() || fread(q.data(), 4, q.size(), f) != q.size()) return 3;
    fclose(f);
    cuLSH::HashTables hashtables;
    cuLSH::SearchTables searchtables;
    if (!hashtables.reset(N, D, L, M, W, Ap.data(), bp.data())) return 4;
    if (!hashtables.index(X.data())) return 5;
    searchtables.reset(&hashtables, K, T);
    if (!searchtables.search(q.data(), Q, X.data())) return 6;
    std::string out = argv[2];
    FILE* o = fopen(out.c_str(), "wb");
    fwrite(searchtables.getKnnIds(), 4, (size_t)Q * K, o);
    fwrite(searchtables.getKnnDistances(), 4, (size_t)Q * K, o);
    for (int l = 0; l < L; ++l) fwrite(searchtables.getQueryBuckets(l), 4, (size_t)Q * T, o);
    unsigned tot[2] = {searchtables.getTotalCandidates_unique(), searchtables.getTotalCandidates_nonUnique()};
    fwrite(tot, 4, 2, o);
    fclose(o);
    cuLSH::SearchTables::timesStruct times;
    searchtables.getTimes(&times);
    printf("selectivity %f nonunique %f distances %f\n", searchtables.getSelectivity(),
           searchtables.getNonUniquePercentage(), times.distances);
    if (!hashtables.save((out + ".index").c_str())) return 7;
    if (hashtables.getBuckets_totalIndices(0)[0] >= (unsigned)N) return 8;
    return 0;
}
"""


def build_dropin(culsh, tmp_path):
    src = tmp_path / "dropin.cpp"
    src.write_text(DROPIN_SRC)
    exe = tmp_path / "dropin"
    libdir = os.path.dirname(culsh.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
           "-L", libdir, "-lculsh", f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True)
    return exe


def test_dropin_header_compiles_and_links(culsh, tmp_path):
    exe = build_dropin(culsh, tmp_path)
    assert exe.exists()


def test_cli_arguments_and_missing_file(culsh):
    """The command-line program keeps the reference demo's contract
    (cuLSH_main.cu:23-32): a usage message and status 0 without exactly nine
    arguments, status 1 for a file that cannot be opened or read. None of
    these paths touches the GPU."""
    from culsh_gb300 import _build
    cli = _build.build_cli()
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 0 and "while 9 are required" in r.stdout
    assert "[filename] [D] [N] [L] [M] [W] [Q] [K] [T]" in r.stdout
    r = subprocess.run([cli, "/nonexistent/data.bin", "4", "10", "1", "2", "1.0", "2", "1", "1"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "Could not open file" in r.stdout


def test_cli_short_file_and_bad_sizes(culsh, tmp_path):
    from culsh_gb300 import _build
    cli = _build.build_cli()
    f = tmp_path / "short.bin"
    np.zeros(10, np.float32).tofile(f)
    r = subprocess.run([cli, str(f), "4", "10", "1", "2", "1.0", "2", "1", "1"], capture_output=True, text=True)
    assert r.returncode == 1 and "Could not load data matrix" in r.stdout
    r = subprocess.run([cli, str(f), "4", "2", "1", "2", "1.0", "3", "1", "1"], capture_output=True, text=True)
    assert r.returncode == 1 and "Invalid sizes" in r.stdout


@pytest.mark.parametrize("cname,pyname", [("culsh_times", "_Times"), ("culsh_index_profile", "_IndexProfile"),
                                          ("culsh_tuning", "_Tuning"), ("culsh_search_profile", "_Profile"),
                                          ("culsh_server_config", "_ServerConfig"),
                                          ("culsh_server_stats", "_ServerStats")])
def test_ctypes_mirrors_match_the_header(culsh, cname, pyname, tmp_path):
    """Every ctypes structure of the Python mirror has the C struct's size and,
    field by field, its offsets and sizes (a C program compiled against
    include/culsh.h prints them)."""
    import ctypes
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    py = getattr(culsh, pyname)
    fields = [f[0] for f in py._fields_]
    lines = [f'printf("size %zu\\n", sizeof({cname}));']
    for f in fields:
        lines.append(f'printf("{f} %zu %zu\\n", offsetof({cname}, {f}), sizeof((({cname}*)0)->{f}));')
    src = tmp_path / "layout.c"
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"culsh.h\"\nint main(void) {\n" +
                   "\n".join("    " + l for l in lines) + "\n    return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    assert out[0] == f"size {ctypes.sizeof(py)}", (cname, out[0], ctypes.sizeof(py))
    for line, f in zip(out[1:], fields):
        name, off, size = line.split()
        d = getattr(py, f)
        assert (name, int(off), int(size)) == (f, d.offset, d.size), (cname, line, d.offset, d.size)


DROPIN_LOAD_SRC = r"""
#include <cstdio>
#include "cuLSH.h"
// argv[1]: an index file; argv[2]: the getters' arrays, written in the file's
// own order; argv[3]: where save() writes the index again.
int main(int argc, char** argv) {
    if (argc != 4) return 2;
    cuLSH::HashTables ht;
    if (ht.reset("/nonexistent/missing.index")) return 3;   // must fail, with the message on stdout
    if (!ht.reset(argv[1])) return 4;
    const int N = ht.getN(), D = ht.getD(), L = ht.getL(), M = ht.getM();
    const float W = ht.getW();
    FILE* o = fopen(argv[2], "wb");
    const int hdr[4] = {N, D, L, M};
    fwrite(hdr, 4, 4, o);
    fwrite(&W, 4, 1, o);
    for (int l = 0; l < L; ++l) {
        fwrite(ht.getA(l), 4, (size_t)D * M, o);
        fwrite(ht.getb(l), 4, (size_t)M, o);
    }
    fwrite(ht.getBuckets(), 4, (size_t)L, o);
    for (int l = 0; l < L; ++l) {
        const unsigned B = ht.getBuckets(l);
        fwrite(ht.getBuckets_totalIndices(l), 4, (size_t)N, o);
        fwrite(ht.getBuckets_startingIndices(l), 4, B, o);
        fwrite(ht.getBuckets_sizes(l), 4, B, o);
        fwrite(ht.getBuckets_codes(l), 4, (size_t)B * M, o);
    }
    fclose(o);
    if (ht.getA(L) || ht.getBuckets_totalIndices(-1)) return 5;   // out-of-range tables read as null
    if (!ht.save(argv[3])) return 6;
    return 0;
}
"""


def test_dropin_header_load_getters_save_without_gpu(culsh, tmp_path):
    """The C++ drop-in (include/cuLSH.h) on the CPU: reset(file) of a missing
    file returns false and prints the error on stdout; reset(file) of the
    oracle's index file fills every getter, whose arrays written in the file's
    order give the file back byte for byte, as does save(); out-of-range
    tables read as null."""
    src = tmp_path / "dropin_load.cpp"
    src.write_text(DROPIN_LOAD_SRC)
    exe = tmp_path / "dropin_load"
    libdir = os.path.dirname(culsh.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-lculsh", f"-Wl,-rpath,{libdir}"], check=True)
    dump, saved = tmp_path / "getters.bin", tmp_path / "saved.index"
    r = subprocess.run([str(exe), INDEX_BIN, str(dump), str(saved)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.startswith("[Error @ ") and "missing.index" in r.stdout, r.stdout
    original = open(INDEX_BIN, "rb").read()
    assert dump.read_bytes() == original
    assert saved.read_bytes() == original
    c = load_case("odd_d13")
    L, M, D = c["A"].shape
    hdr = np.frombuffer(original[:16], np.int32)
    assert tuple(hdr) == (c["X"].shape[0], D, L, M)

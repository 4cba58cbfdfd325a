"""The reference-side binding: heFFTe's own classes and C API on this library.

The binding header (include/heffte_backend_gb300.h) and the location-layer
shim (heffte_gb300/integration/heffte_backend_gb300_location.cpp) are compiled
with the reference's headers and its src/heffte_plan_logic.cpp,
heffte_reshape3d.cpp and heffte_compute_transform.cpp (Heffte_ENABLE_CUDA,
single-rank MPI stand-in), linked to libheffte_gb300.so, and

* (CPU) heffte::fft3d<gb300>, fft3d_r2c<gb300> and rtransform<gb300_cos|cos1>
  plans are built on MPI_COMM_SELF (plan construction touches no GPU), and the
  DCT-I scale after the one-line edit of the reference's scale table;
* (GPU) the same classes run forward / backward through the reference's
  compute_transform, reshape3d_transpose (use_reorder) and the executors'
  real-input overloads, on the seeded fixtures the reference itself computed
  (tests/golden/seeded.npz) and on extra boxes against the FP64 oracle
  (tests/binding/run_jobs.cpp);
* (GPU) the reference's C API with the new backend id: heffte_c.cpp and
  heffte_c_defines.h with the maintainer's edit, driven from C
  (tests/binding/c_api.c).

The reference tree is $HEFFTE_REFERENCE_DIR, else a folder named "reference"
beside this repository; a host without it (the GPU host) uses the copy that
`make -C oracle/ref stage` leaves in oracle/_ref/reference (git-ignored).
"""
import os
import re
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import heffte_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME") or "/usr/local/cuda"
BINDING = os.path.join(ROOT, "tests", "binding")


def _reference_dir():
    env = os.environ.get("HEFFTE_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")
    for cand in (env, os.path.join(ROOT, "oracle", "_ref", "reference")):
        if os.path.isfile(os.path.join(cand, "include", "heffte.h")) and \
                os.path.isfile(os.path.join(cand, "src", "heffte_compute_transform.cpp")):
            return cand
    return None


REF = _reference_dir()

pytestmark = pytest.mark.skipif(REF is None or shutil.which("g++") is None,
                                reason="reference tree (or its staged copy) or g++ not available")

REF_SRCS = ["heffte_plan_logic.cpp", "heffte_reshape3d.cpp", "heffte_compute_transform.cpp"]

MAIN = r'''
#include "heffte.h"
#include "heffte_backend_gb300.h"
#include <cstdio>
using namespace heffte;
int main(){
    box3d<> world({0, 0, 0}, {63, 31, 15});
    fft3d<backend::gb300> c2c(world, world, MPI_COMM_SELF);
    fft3d_r2c<backend::gb300> r2c(world, world.r2c(0), 0, MPI_COMM_SELF);
    rtransform<backend::gb300_cos> cosx(world, world, MPI_COMM_SELF);
    box3d<> world1({0, 0, 0}, {64, 32, 16});   // DCT-I lengths 65, 33, 17: FFTs of 128, 64, 32
    rtransform<backend::gb300_cos1> cos1x(world1, world1, MPI_COMM_SELF);
    plan_options reorder = default_options<backend::gb300>();
    reorder.use_reorder = true;
    fft3d<backend::gb300> c2c_reorder(world, box3d<>({0, 0, 0}, {63, 31, 15}, {2, 1, 0}), MPI_COMM_SELF, reorder);
    std::printf("%s %lld %lld %lld %lld %lld %zu %.17g %.17g\n", backend::name<backend::gb300>().c_str(),
                c2c.size_inbox(), c2c.size_outbox(), r2c.size_outbox(), cosx.size_inbox(),
                c2c_reorder.size_outbox(), c2c_reorder.size_workspace(), cosx.get_scale_factor(scale::full),
                cos1x.get_scale_factor(scale::full));
    return 0;
}
'''


# The edit a maintainer makes for the DCT-I tag: the DCT-I branch of the
# scale table keys on tag identity (include/heffte_fft3d.h:643-645), so the tag
# is declared where the other tags are (a forward declaration is enough) and
# added to that branch.
COS1_LIST = "std::is_same<backend_tag, backend::stock_cos1>::value){"
COS1_LIST_PATCHED = ("std::is_same<backend_tag, backend::stock_cos1>::value or\n"
                     "                     std::is_same<backend_tag, backend::gb300_cos1>::value){")
COS1_DECL = "namespace heffte { namespace backend { struct gb300_cos1; } }\n"


def _patched_include(tmp, replacements):
    """The reference headers by symlink (quoted includes resolve next to the
    including file), the files in `replacements` (name -> text) written out."""
    inc = os.path.join(tmp, "patched")
    os.makedirs(inc)
    src_inc = os.path.join(REF, "include")
    for entry in os.listdir(src_inc):
        if entry not in replacements:
            os.symlink(os.path.join(src_inc, entry), os.path.join(inc, entry))
    for name, text in replacements.items():
        with open(os.path.join(inc, name), "w") as f:
            f.write(text)
    return inc


def _compile(gb, tmp, sources, ref_include=None, defines=(), libs=(), c_sources=()):
    lib_dir = os.path.dirname(gb.library_path)
    inc = ["-I" + os.path.join(ROOT, "oracle", "ref"), "-I" + (ref_include or os.path.join(REF, "include")),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CUDA, "include")]
    objs = []
    for i, c in enumerate(c_sources):
        o = os.path.join(tmp, f"c{i}.o")
        r = subprocess.run(["gcc", "-std=gnu11", "-O0", "-w", "-c", c, "-o", o] + list(defines) + inc,
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]
        objs.append(o)
    exe = os.path.join(tmp, "prog")
    cmd = ["g++", "-std=c++17", "-O0", "-w", "-DHeffte_ENABLE_CUDA", "-DHeffte_ENABLE_GPU"] + list(defines) + inc + \
          list(sources) + objs + \
          [os.path.join(ROOT, "heffte_gb300", "integration", "heffte_backend_gb300_location.cpp")] + \
          [os.path.join(REF, "src", s) for s in REF_SRCS] + \
          ["-L" + lib_dir, "-lheffte_gb300", "-Wl,-rpath," + lib_dir,
           "-L" + os.path.join(CUDA, "lib64"), "-lcudart"] + list(libs) + \
          ["-Wl,-rpath," + os.path.join(CUDA, "lib64"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


def _build_and_run(gb, tmp, ref_include=None):
    main = os.path.join(tmp, "main.cpp")
    with open(main, "w") as f:
        f.write(MAIN)
    exe = _compile(gb, tmp, [main], ref_include)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    return out.stdout.split()


def test_reference_fft3d_plans_with_gb300_tags(gb):
    with tempfile.TemporaryDirectory() as tmp:
        name, nin, nout, nr2c, ncos, nreo, wreo, scale, scale1 = _build_and_run(gb, tmp)
    assert name == "gb300"
    assert int(nin) == int(nout) == 64 * 32 * 16
    assert int(nr2c) == 33 * 32 * 16
    assert int(ncos) == 64 * 32 * 16 and int(nreo) == 64 * 32 * 16
    assert int(wreo) > 0  # the reordering plan carries transposes and needs a workspace
    assert abs(float(scale) - 1.0 / (64 * 64 * 32 * 16)) < 1e-20
    # unedited reference: a new cos1 tag falls into the default 1/(64 N) branch
    assert abs(float(scale1) - 1.0 / (64 * 65 * 33 * 17)) < 1e-20


def _fft3d_h_with_cos1_edit():
    with open(os.path.join(REF, "include", "heffte_fft3d.h")) as f:
        text = f.read()
    assert text.count(COS1_LIST) == 1
    return COS1_DECL + text.replace(COS1_LIST, COS1_LIST_PATCHED)


def test_reference_cos1_scale_after_the_one_line_edit(gb):
    """With gb300_cos1 added to the DCT-I branch of the scale table the
    reference gives 1/(64 prod(n - 1)), the value this library uses."""
    with tempfile.TemporaryDirectory() as tmp:
        inc = _patched_include(tmp, {"heffte_fft3d.h": _fft3d_h_with_cos1_edit()})
        *_, scale1 = _build_and_run(gb, tmp, inc)
    assert abs(float(scale1) - 1.0 / (64 * 64 * 32 * 16)) < 1e-20


# ---------------------------------------------------------------------------
# the classes running on the GPU
# ---------------------------------------------------------------------------
R2R_NAMES = {0: "cos", 1: "sin", 2: "cos1"}
FTOL = {0: 1e-6, 1: 1e-12}          # against the FP64 oracle
RTOL = {0: 5e-6, 1: 1e-12}          # against the reference's own outputs (stock<float> for float)


def _cdt(prec):
    return np.complex64 if prec == 0 else np.complex128


def _rdt(prec):
    return np.float32 if prec == 0 else np.float64


def _job_line(kind, prec, reorder, size, io, oo, r2c_dir, api, prefix):
    return " ".join(str(v) for v in [kind, prec, reorder, *size, *io, *oo, r2c_dir, api, prefix])


@pytest.mark.gpu
def test_reference_classes_run_on_gb300(gb, golden, report):
    """heffte::fft3d / fft3d_r2c / rtransform<gb300*> forward and backward on
    the GPU through the reference's own compute_transform: every seeded
    fixture of the reference, with use_reorder off and on, through the pointer
    API with and without a workspace, the vector API and a user stream; plus
    in-place c2c and fft3d with real input (the executor's real overloads)."""
    g = golden["seeded"]
    jobs, checks = [], []
    with tempfile.TemporaryDirectory() as tmp:
        exe = _compile(gb, tmp, [os.path.join(BINDING, "run_jobs.cpp")])
        k = 0
        for m in g["meta"]:
            key = str(m["key"])
            size = (int(m["n0"]), int(m["n1"]), int(m["n2"]))
            io = (int(m["io0"]), int(m["io1"]), int(m["io2"]))
            oo = (int(m["oo0"]), int(m["oo1"]), int(m["oo2"]))
            prec = int(m["prec"])
            kind = str(m["kind"])
            if kind == "r2r":
                kind = R2R_NAMES[int(m["r2r_kind"])]
            x, fwd_ref, bwd_ref = g[key + "_in"], g[key + "_fwd"], g[key + "_bwd"]
            in_dt = _cdt(prec) if kind == "c2c" else _rdt(prec)
            out_dt = _cdt(prec) if kind in ("c2c", "r2c") else _rdt(prec)
            for reorder in (0, 1):
                api = (0, 1, 2, 4)[k % 4]
                k += 1
                prefix = os.path.join(tmp, f"{key}_r{reorder}")
                np.asarray(x, dtype=in_dt).tofile(prefix + "_in.bin")
                np.asarray(fwd_ref, dtype=out_dt).tofile(prefix + "_fin.bin")
                r2c_dir = int(m["r2c_dir"]) if kind == "r2c" else 0
                jobs.append(_job_line(kind, prec, reorder, size, io, oo, r2c_dir, api, prefix))
                # the unedited reference scales a new cos1 tag by 1/(64 N), not
                # 1/(64 prod(n - 1)): compare the backward result rescaled
                bscale = (np.prod(size) / np.prod([s - 1 for s in size])) if kind == "cos1" else 1.0
                checks.append((f"{key} reorder={reorder} api={api}", prefix, prec, out_dt, in_dt,
                               fwd_ref, bwd_ref, bscale))
        # fft3d with real input and output (the executor's convert overloads),
        # and in-place c2c, on a box that is not in the fixtures
        rng = np.random.default_rng(77)
        size = (12, 10, 9)
        n = int(np.prod(size))
        for prec in (0, 1):
            xr = rng.standard_normal(n)
            spec = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
            prefix = os.path.join(tmp, f"real_p{prec}")
            xr.astype(_rdt(prec)).tofile(prefix + "_in.bin")
            spec.astype(_cdt(prec)).tofile(prefix + "_fin.bin")
            jobs.append(_job_line("real", prec, prec, size, (0, 1, 2), (0, 1, 2), 0, 0, prefix))
            checks.append((f"real-input fft3d prec={prec}", prefix, prec, _cdt(prec), _rdt(prec),
                           O.fft3d_c2c(xr, size), O.fft3d_c2c(spec, size, direction=1, scaling=O.SCALE_FULL).real,
                           1.0))
            xc = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
            prefix = os.path.join(tmp, f"inplace_p{prec}")
            xc.astype(_cdt(prec)).tofile(prefix + "_in.bin")
            spec.astype(_cdt(prec)).tofile(prefix + "_fin.bin")
            jobs.append(_job_line("c2c", prec, 1 - prec, size, (0, 1, 2), (0, 1, 2), 0, 3, prefix))
            checks.append((f"in-place c2c prec={prec}", prefix, prec, _cdt(prec), _cdt(prec),
                           O.fft3d_c2c(xc, size), O.fft3d_c2c(spec, size, direction=1, scaling=O.SCALE_FULL), 1.0))
        jobfile = os.path.join(tmp, "jobs.txt")
        with open(jobfile, "w") as f:
            f.write("\n".join(jobs) + "\n")
        out = subprocess.run([exe, jobfile], capture_output=True, text=True, timeout=600)
        assert out.returncode == 0, out.stderr[-4000:]
        worst = {0: 0.0, 1: 0.0}
        failed = []
        for label, prefix, prec, out_dt, in_dt, fwd_ref, bwd_ref, bscale in checks:
            fwd = np.fromfile(prefix + "_fwd.bin", dtype=out_dt)
            bwd = np.fromfile(prefix + "_bwd.bin", dtype=in_dt) * bscale
            ef, eb = O.rel_l2(fwd, fwd_ref), O.rel_l2(bwd, bwd_ref)
            worst[prec] = max(worst[prec], ef, eb)
            if not (ef < RTOL[prec] and eb < RTOL[prec]):
                failed.append((label, ef, eb))
        assert not failed, failed
    report.append(f"reference classes on gb300: {len(jobs)} jobs, worst rel-L2 float {worst[0]:.2e}, "
                  f"double {worst[1]:.2e}")


# ---------------------------------------------------------------------------
# the reference's C API with the new backend id
# ---------------------------------------------------------------------------
C_DEFINES_ANCHOR = "#define Heffte_SUCCESS 0"
C_DEFINES_ADD = ("#ifdef Heffte_ENABLE_GB300\n"
                 "/*! \\brief Set the use of the GB300 backend. */\n"
                 "#define Heffte_BACKEND_GB300 20\n"
                 "#endif\n\n")


def _c_api_with_gb300_id(text):
    """The maintainer's edit of src/heffte_c.cpp: include the binding header
    and, next to every cuFFT case of the id dispatch, the same case for the
    GB300 id and tag."""
    text = text.replace('#include "heffte_c_defines.h"\n',
                        '#include "heffte_c_defines.h"\n#ifdef Heffte_ENABLE_GB300\n'
                        '#include "heffte_backend_gb300.h"\n#endif\n', 1)
    blocks = re.findall(r"[ \t]*#ifdef Heffte_ENABLE_CUDA\n(?:(?!#endif).)*?Heffte_BACKEND_CUFFT(?:(?!#endif).)*?#endif\n",
                        text, flags=re.S)
    assert len(blocks) >= 8, len(blocks)
    for b in set(blocks):
        twin = (b.replace("Heffte_ENABLE_CUDA", "Heffte_ENABLE_GB300").replace("Heffte_BACKEND_CUFFT", "Heffte_BACKEND_GB300")
                 .replace("backend::cufft", "backend::gb300"))
        text = text.replace(b, b + twin)
    return text


@pytest.mark.gpu
def test_reference_c_api_with_gb300_backend_id(gb, report):
    """heffte_plan_create / heffte_plan_create_r2c (Heffte_BACKEND_GB300),
    heffte_forward_{c2c,z2z,s2c,d2z} and heffte_backward_* from C, against
    the FP64 oracle."""
    libcufft = os.path.join(CUDA, "lib64", "libcufft.so")
    if not os.path.exists(libcufft):
        pytest.skip("the unedited cuFFT cases of heffte_c.cpp need libcufft to link")
    with open(os.path.join(REF, "include", "heffte_c_defines.h")) as f:
        defines = f.read()
    assert defines.count(C_DEFINES_ANCHOR) == 1
    with open(os.path.join(REF, "src", "heffte_c.cpp")) as f:
        capi = f.read()
    rng = np.random.default_rng(5)
    size = (20, 18, 12)
    n = int(np.prod(size))
    with tempfile.TemporaryDirectory() as tmp:
        inc = _patched_include(tmp, {"heffte_c_defines.h": defines.replace(C_DEFINES_ANCHOR,
                                                                           C_DEFINES_ADD + C_DEFINES_ANCHOR)})
        src = os.path.join(tmp, "heffte_c.cpp")
        with open(src, "w") as f:
            f.write(_c_api_with_gb300_id(capi))
        exe = _compile(gb, tmp, [src], inc, defines=["-DHeffte_ENABLE_GB300"],
                       libs=["-lcufft"], c_sources=[os.path.join(BINDING, "c_api.c")])
        worst = 0.0
        for prec in (0, 1):
            for r2c in (0, 1):
                prefix = os.path.join(tmp, f"c{prec}{r2c}")
                nc = (size[0] // 2 + 1) * size[1] * size[2] if r2c else n
                x = rng.standard_normal(n) if r2c else rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
                if r2c:
                    # a valid half spectrum: the r2c transform of a real box
                    spec = O.fft3d_r2c(rng.standard_normal(n), size, 0)
                else:
                    spec = rng.uniform(-1, 1, nc) + 1j * rng.uniform(-1, 1, nc)
                (x.astype(_rdt(prec)) if r2c else x.astype(_cdt(prec))).tofile(prefix + "_in.bin")
                spec.astype(_cdt(prec)).tofile(prefix + "_fin.bin")
                out = subprocess.run([exe, str(prec), str(r2c), *map(str, size), prefix], capture_output=True,
                                     text=True, timeout=300)
                assert out.returncode == 0, out.stderr[-4000:]
                backend, is_r2c, nin, nout = map(int, out.stdout.split())
                assert backend == 20 and is_r2c == r2c and nin == n and nout == nc
                fwd = np.fromfile(prefix + "_fwd.bin", dtype=_cdt(prec))
                bwd = np.fromfile(prefix + "_bwd.bin", dtype=_rdt(prec) if r2c else _cdt(prec))
                if r2c:
                    want_f = O.fft3d_r2c(x, size, 0)
                    want_b = O.fft3d_c2r(spec, size, 0, scaling=O.SCALE_FULL)
                else:
                    want_f = O.fft3d_c2c(x, size)
                    want_b = O.fft3d_c2c(spec, size, direction=1, scaling=O.SCALE_FULL)
                ef, eb = O.rel_l2(fwd, want_f), O.rel_l2(bwd, want_b)
                assert ef < FTOL[prec] and eb < FTOL[prec], (prec, r2c, ef, eb)
                worst = max(worst, ef if prec == 1 else 0.0, eb if prec == 1 else 0.0)
    report.append(f"reference C API with Heffte_BACKEND_GB300: c2c/z2z/s2c/d2z ok (double worst rel-L2 {worst:.2e})")

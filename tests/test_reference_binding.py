"""The reference-side binding compiles against the reference's own headers and
plans through heFFTe's own fft3d / fft3d_r2c / rtransform classes.

Compiles include/heffte_backend_gb300.h and the location-layer shim
(heffte_gb300/integration/heffte_backend_gb300_location.cpp) together with
the reference's src/*.cpp (Heffte_ENABLE_CUDA, single-rank MPI stand-in),
links libheffte_gb300.so and runs a program that builds heffte::fft3d<gb300>,
fft3d_r2c<gb300> and rtransform<gb300_cos> plans on MPI_COMM_SELF (plan
construction touches no GPU).  Needs the reference tree, so it runs where the
reference is mounted and is skipped elsewhere.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference heFFTe tree: $HEFFTE_REFERENCE_DIR, else "reference" beside this repository
REF = os.environ.get("HEFFTE_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")
CUDA = "/usr/local/cuda"

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include")) or shutil.which("g++") is None,
                                reason="reference tree or g++ not available")

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


def _build_and_run(gb, tmp, ref_include=None):
    lib_dir = os.path.dirname(gb.library_path)
    main = os.path.join(tmp, "main.cpp")
    with open(main, "w") as f:
        f.write(MAIN)
    exe = os.path.join(tmp, "binding")
    inc = ["-I" + os.path.join(ROOT, "oracle", "ref"), "-I" + (ref_include or os.path.join(REF, "include")),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CUDA, "include")]
    cmd = ["g++", "-std=c++17", "-O0", "-w", "-DHeffte_ENABLE_CUDA", "-DHeffte_ENABLE_GPU"] + inc + [
           main, os.path.join(ROOT, "heffte_gb300", "integration", "heffte_backend_gb300_location.cpp"),
           os.path.join(REF, "src", "heffte_plan_logic.cpp"), os.path.join(REF, "src", "heffte_reshape3d.cpp"),
           os.path.join(REF, "src", "heffte_compute_transform.cpp"),
           "-L" + lib_dir, "-lheffte_gb300", "-Wl,-rpath," + lib_dir,
           "-L" + os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(CUDA, "lib64"),
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
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


def test_reference_cos1_scale_after_the_one_line_edit(gb):
    """With gb300_cos1 added to the DCT-I branch of the scale table the
    reference gives 1/(64 prod(n - 1)), the value this library uses."""
    with open(os.path.join(REF, "include", "heffte_fft3d.h")) as f:
        text = f.read()
    assert text.count(COS1_LIST) == 1
    with tempfile.TemporaryDirectory() as tmp:
        # the reference headers by symlink (quoted includes resolve next to the
        # including file), heffte_fft3d.h with the edit
        inc = os.path.join(tmp, "patched")
        os.makedirs(inc)
        src_inc = os.path.join(REF, "include")
        for entry in os.listdir(src_inc):
            if entry != "heffte_fft3d.h":
                os.symlink(os.path.join(src_inc, entry), os.path.join(inc, entry))
        with open(os.path.join(inc, "heffte_fft3d.h"), "w") as f:
            f.write(COS1_DECL + text.replace(COS1_LIST, COS1_LIST_PATCHED))
        *_, scale1 = _build_and_run(gb, tmp, inc)
    assert abs(float(scale1) - 1.0 / (64 * 64 * 32 * 16)) < 1e-20

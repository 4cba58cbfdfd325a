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
REF = "/root/reference"
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
    plan_options reorder = default_options<backend::gb300>();
    reorder.use_reorder = true;
    fft3d<backend::gb300> c2c_reorder(world, box3d<>({0, 0, 0}, {63, 31, 15}, {2, 1, 0}), MPI_COMM_SELF, reorder);
    std::printf("%s %lld %lld %lld %lld %lld %zu %.17g\n", backend::name<backend::gb300>().c_str(),
                c2c.size_inbox(), c2c.size_outbox(), r2c.size_outbox(), cosx.size_inbox(),
                c2c_reorder.size_outbox(), c2c_reorder.size_workspace(), cosx.get_scale_factor(scale::full));
    return 0;
}
'''


def test_reference_fft3d_plans_with_gb300_tags(gb):
    lib_dir = os.path.dirname(gb.library_path)
    with tempfile.TemporaryDirectory() as tmp:
        main = os.path.join(tmp, "main.cpp")
        with open(main, "w") as f:
            f.write(MAIN)
        exe = os.path.join(tmp, "binding")
        cmd = ["g++", "-std=c++17", "-O0", "-w", "-DHeffte_ENABLE_CUDA", "-DHeffte_ENABLE_GPU",
               "-I" + os.path.join(ROOT, "oracle", "ref"), "-I" + os.path.join(REF, "include"),
               "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CUDA, "include"),
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
        name, nin, nout, nr2c, ncos, nreo, wreo, scale = out.stdout.split()
        assert name == "gb300"
        assert int(nin) == int(nout) == 64 * 32 * 16
        assert int(nr2c) == 33 * 32 * 16
        assert int(ncos) == 64 * 32 * 16 and int(nreo) == 64 * 32 * 16
        assert int(wreo) > 0  # the reordering plan carries transposes and needs a workspace
        assert abs(float(scale) - 1.0 / (64 * 64 * 32 * 16)) < 1e-20

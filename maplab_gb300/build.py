"""Builds the native libraries in-tree (maplab_gb300/_build/).

* libmaplab_ba.so  — the CUDA back-end (sm_103a only), C ABI of include/maplab_ba.h, and the
                    host VIMap map-folder reader / exporter of include/maplab_vimap.h
* libmba_synth.so  — host-only synthetic map generator (include/maplab_ba_synth.h)

Each translation unit compiles in its own process so a build takes about as
long as the slowest unit.  No cmake.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")

CUDA_SOURCES = ["mba_api.cu", "kernels_eval.cu", "kernels_inertial.cu", "kernels_solver.cu", "kernels_chain.cu",
                "kernels_gnn.cu", "kernels_gnn_tc.cu", "kernels_pose.cu", "noalloc.cu", "kernels_peak.cu",
                "kernels_border.cu"]
HOST_SOURCES = ["vimap_io.cc"]  # host-only parts of libmaplab_ba.so (g++)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run_parallel(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out.decode(errors="replace")))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("native build failed:\n" + msg)


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose=False, ptxas_verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    # CUDA objects
    cmds, objs = [], []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + headers):
            cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", s, "-o", o]
            if ptxas_verbose:
                cmd += ["-Xptxas", "-v"]
            cmds.append(cmd)
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cc", ".o"))
        objs.append(o)
        if _stale(o, [s] + headers):
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", os.path.join(ROOT, "include"), "-c", s,
                         "-o", o])
    synth_src = os.path.join(CSRC, "synth_map.cc")
    synth_so = os.path.join(BUILD, "libmba_synth.so")
    if _stale(synth_so, [synth_src] + headers):
        cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-o", synth_so, synth_src])
    if cmds:
        if verbose:
            for c in cmds:
                print(" ".join(c))
        _run_parallel(cmds)
    so = os.path.join(BUILD, "libmaplab_ba.so")
    if _stale(so, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", so] + objs + ["-lcudart"]
        if verbose:
            print(" ".join(cmd))
        _run_parallel([cmd])
    return so


if __name__ == "__main__":
    build(verbose=True, ptxas_verbose="-v" in sys.argv)

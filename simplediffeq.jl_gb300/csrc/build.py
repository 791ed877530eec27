#!/usr/bin/env python3
"""Build libgb300ode.so for sm_103a.

Steps:
  1. embed the device headers as C strings for run-time compilation (NVRTC);
  2. write one translation unit per group of ahead-of-time kernels, plus the
     registry the library uses to find them;
  3. compile every translation unit with nvcc in parallel
     (-gencode arch=compute_103a,code=sm_103a --fmad=false) and link.

Outputs go to simplediffeq.jl_gb300/_build/ (objects, generated sources) and
simplediffeq.jl_gb300/lib/ (the shared libraries).
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
CUDA_HOME = os.path.dirname(os.path.dirname(os.path.realpath(NVCC)))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", HERE]

# Kernels compiled ahead of time: (alg, kind, rhs, dim, precision, rhs C++ type).
# Everything else is compiled on first use with NVRTC from the same headers.
ALG = {"rk4": 0, "tsit5": 1, "atsit5": 2, "vern7": 3, "avern7": 4, "vern9": 5, "avern9": 6, "euler": 7}
METHOD = {"rk4": "gbode::MRK4", "tsit5": "gbode::MTsit5", "atsit5": "gbode::MTsit5", "vern7": "gbode::MVern7",
          "avern7": "gbode::MVern7", "vern9": "gbode::MVern9", "avern9": "gbode::MAVern9", "euler": "gbode::MEuler"}
RHS = {"lorenz": 0, "vanderpol": 1, "r3bp": 2, "kuramoto": 3, "linear": 4}
PREC = {"fp64": (0, "gbode::PFP64", "double", "double"), "fp32": (1, "gbode::PFP32", "float", "float"),
        "fp32k": (2, "gbode::PFP32K", "float", "double")}


def rhs_type(rhs, dim, prec):
    _, _, R, T = PREC[prec]
    return {"lorenz": "gbode::RhsLorenz<%s, %s>" % (R, T),
            "vanderpol": "gbode::RhsVanDerPol<%s, %s>" % (R, T),
            "r3bp": "gbode::RhsR3BP<%s, %s>" % (R, T),
            "kuramoto": "gbode::RhsKuramoto<%s, %s, %d>" % (R, T, dim),
            "linear": "gbode::RhsLinear<%s, %s, %d>" % (R, T, dim)}[rhs]


GROUPS = {
    # the ensemble workloads: fixed Tsit5 / adaptive ATsit5 on Lorenz, AVern7 on
    # Van der Pol, AVern9 on the restricted three-body problem, ATsit5 on Kuramoto-12
    "lorenz": [("tsit5", "fixed", "lorenz", 3, "fp64"),
               ("tsit5", "fixedsplit", "lorenz", 3, "fp64"),
               ("atsit5", "plain", "lorenz", 3, "fp64"),
               ("atsit5", "persistent", "lorenz", 3, "fp64")],
    "lorenz_staged": [("atsit5", "staged", "lorenz", 3, "fp64")],
    "vdp": [("avern7", "plain", "vanderpol", 2, "fp64"),
            ("avern7", "persistent", "vanderpol", 2, "fp64")],
    "vdp_staged": [("avern7", "staged", "vanderpol", 2, "fp64")],
    "r3bp64": [("avern9", "plain", "r3bp", 4, "fp64"),
               ("avern9", "persistent", "r3bp", 4, "fp64")],
    "r3bp32": [("avern9", "plain", "r3bp", 4, "fp32k"),
               ("avern9", "persistent", "r3bp", 4, "fp32k")],
    "kuramoto": [("atsit5", "plain", "kuramoto", 12, "fp64"),
                 ("atsit5", "persistent", "kuramoto", 12, "fp64")],
    "kuramoto_staged": [("atsit5", "staged", "kuramoto", 12, "fp64")],
}


# Launch shape of a group's kernels (threads per block, staging-ring bytes per
# warp), where it is not the default 128 / 12 KB: the staged kernels take the
# shape the autotuner picks on the benchmark workloads (a ring that holds a
# round plus a step's worth of new jobs, at no cost in occupancy); Kuramoto-12's
# 804-byte jobs take one-warp blocks with a ring of exactly one round (32 jobs),
# eight warps per SM.
SHAPES = {"lorenz_staged": (64, 24576), "vdp_staged": (64, 24576), "kuramoto_staged": (32, 26112)}


def kname(alg, kind, rhs, dim, prec):
    return "gbode_%s_%s_%s%d_%s" % (alg, kind, rhs, dim, prec)


def write_if_changed(path, text):
    if os.path.exists(path) and open(path).read() == text:
        return
    with open(path, "w") as f:
        f.write(text)


def gen_sources():
    os.makedirs(BUILD, exist_ok=True)
    # 1. embedded headers
    parts = ["/* generated by build.py: device headers for NVRTC */\n"]
    for fname, var in (("ode_solver.cuh", "kSrc_ode_solver_cuh"), ("ode_kparams.h", "kSrc_ode_kparams_h"),
                       ("tableaus.h", "kSrc_tableaus_h"), ("sde_solver.cuh", "kSrc_sde_solver_cuh"),
                       ("log_table.h", "kSrc_log_table_h"), ("exp_table.h", "kSrc_exp_table_h"),
                       ("ds_table.h", "kSrc_ds_table_h"), ("bitops.h", "kSrc_bitops_h"),
                       ("crpow.h", "kSrc_crpow_h"), ("crpow_table.h", "kSrc_crpow_table_h")):
        text = open(os.path.join(HERE, fname)).read()
        assert ")GBSRC\"" not in text
        parts.append('static const char* %s = R"GBSRC(%s)GBSRC";\n' % (var, text))
    write_if_changed(os.path.join(BUILD, "embedded_src.inc"), "".join(parts))
    # 2. ahead-of-time kernels and their registry
    decl, entries, tus = [], [], []
    for g, items in GROUPS.items():
        block, ring = SHAPES.get(g, (128, 12288))
        lines = ["/* generated by build.py: ahead-of-time kernels, group %s */\n" % g,
                 "#define GBODE_BLOCK %d\n#define GBODE_STAGE_BYTES %d\n" % (block, ring),
                 "#define GBODE_CTRL_DS 1 /* the default error norm and controller (ODE_CTRL_DS) */\n",
                 '#include "ode_solver.cuh"\n']
        for i, (alg, kind, rhs, dim, prec) in enumerate(items):
            t = "RHS_%s_%d" % (g, i)
            lines.append("typedef %s %s;\n" % (rhs_type(rhs, dim, prec), t))
            lines.append("GBODE_ENTRY(%s, %s, %s, %s, %s)\n" % (kname(alg, kind, rhs, dim, prec), kind,
                                                               METHOD[alg], PREC[prec][1], t))
            decl.append('extern "C" __global__ void %s(gbode::KParams);\n' % kname(alg, kind, rhs, dim, prec))
            entries.append('  {%d, "%s", %d, %d, %d, (const void*)%s, %d, %d},\n' % (
                ALG[alg], kind, RHS[rhs], dim, PREC[prec][0], kname(alg, kind, rhs, dim, prec), block, ring))
        path = os.path.join(BUILD, "kern_%s.cu" % g)
        write_if_changed(path, "".join(lines))
        tus.append(path)
    reg = ["/* generated by build.py: kernels compiled ahead of time */\n",
           "struct AotEntry { int alg; const char* kind; int rhs; int dim; int precision; const void* fn; int block; "
           "int stage; };\n"]
    reg += decl
    reg.append("static const AotEntry kAotEntries[] = {\n")
    reg += entries
    reg.append("};\n")
    write_if_changed(os.path.join(BUILD, "aot_registry.inc"), "".join(reg))
    return tus


def _deps_hash(src, extra):
    h = hashlib.sha256()
    for p in [src] + extra:
        h.update(open(p, "rb").read())
    h.update(" ".join(COMMON + ARCH).encode())
    return h.hexdigest()


def compile_one(src, obj, extra_deps, flags=()):
    stamp = obj + ".hash"
    digest = _deps_hash(src, extra_deps)
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == digest:
        return obj, None
    cmd = [NVCC] + ARCH + COMMON + list(flags) + ["-I", BUILD, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "%s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr)
    open(stamp, "w").write(digest)
    return obj, (r.stderr if "warning" in r.stderr else None)


def build(verbose=False, jobs=None):
    tus = gen_sources()
    os.makedirs(LIB, exist_ok=True)
    headers = [os.path.join(HERE, f) for f in ("ode_solver.cuh", "ode_kparams.h", "tableaus.h", "ode_host.h",
                                               "jlrange.h", "sde_solver.cuh", "log_table.h", "exp_table.h",
                                               "ds_table.h", "bitops.h", "crpow.h", "crpow_table.h")] + [
        os.path.join(PKG, "..", "include", "gb300ode.h")]
    host_tus = [os.path.join(HERE, f) for f in ("ode_capi.cu", "learn.cu", "noalloc.cu", "sde_capi.cu")]
    gen = [os.path.join(BUILD, "aot_registry.inc"), os.path.join(BUILD, "embedded_src.inc")]
    jobs_list = []
    for src in tus + host_tus:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        jobs_list.append((src, obj, headers + gen))
    errors = []
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count()) as ex:
        futs = [ex.submit(compile_one, s, o, d) for s, o, d in jobs_list]
        for f in futs:
            obj, msg = f.result()
            if msg:
                (errors if not os.path.exists(obj + ".hash") or "error" in msg else []).append(msg)
                if verbose:
                    print(msg, file=sys.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    objs = [o for s, o, d in jobs_list]
    out = os.path.join(LIB, "libgb300ode.so")
    link = [NVCC] + ARCH + ["-shared", "-o", out] + objs + ["-ldl"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))

"""Build the CUDA library ``libgaussium_gb300.so`` in-tree for sm_103a.

Steps: run the class generator (csrc/gen_eri.py) and the Boys-table generator
(csrc/boys_table_gen.c, compiled with gcc) into ``_build/gen``, write one translation unit
per angular-momentum class, compile all of them in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a``) and link them with the C-ABI file
``csrc/capi.cu``.  Objects are rebuilt only when their inputs change.
"""
import concurrent.futures as cf
import hashlib
import json
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
# GS_BUILD_DIR / GS_LIB_PATH / GS_NVCC_EXTRA let a tuning sweep build variants side by side
BUILD = os.environ.get("GS_BUILD_DIR", os.path.join(PKG, "_build"))
GEN = os.path.join(BUILD, "gen")
LIB = os.environ.get("GS_LIB_PATH", os.path.join(PKG, "libgaussium_gb300.so"))
HOSTCHECK = os.path.join(BUILD, "libhostcheck.so")
LMAX = 2
# Kernel forms per class (csrc/eri_launch.cuh dispatches): classes with total angular
# momentum L <= THREAD64_MAX / THREAD32_MAX get the one-thread-per-quartet kernel
# (csrc/eri_kernels.cuh) in FP64 / FP32, classes with L >= WIDE_PROG_MIN (FP64) or
# L >= WIDE32_FROM (FP32) the warp-cooperative kernel (csrc/eri_wide.cuh).  Where a class
# has both, WIDE64_MIN / WIDE32_MIN set the default and gs_set_class_variant (the
# autotuner) can choose per class at run time.
WIDE64_MIN = int(os.environ.get("GS_WIDE64_MIN", "3"))
WIDE32_MIN = int(os.environ.get("GS_WIDE32_MIN", "8"))
THREAD64_MAX = int(os.environ.get("GS_THREAD64_MAX", "4"))
THREAD32_MAX = 7
WIDE32_FROM = 0
WIDE_PROG_MIN = 0          # classes that get generated warp programs (all: the heavy
                           # quartets of a thread-form class run in the warp form)
GRAD_THREAD_LMAX = 3       # gradient classes with a thread-per-quartet form (gen_grad.py)

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                  "--expt-relaxed-constexpr", "-I", CSRC, "-I", GEN] + \
    os.environ.get("GS_NVCC_EXTRA", "").split()


def _run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _digest(paths, extra=""):
    h = hashlib.sha256(extra.encode())
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def classes():
    sys.path.insert(0, CSRC)
    try:
        import gen_eri
    finally:
        sys.path.pop(0)
    return gen_eri.canonical_classes(LMAX)


def generate():
    os.makedirs(GEN, exist_ok=True)
    _run([sys.executable, os.path.join(CSRC, "gen_eri.py"), GEN, str(LMAX)])
    _run([sys.executable, os.path.join(CSRC, "gen_grad.py"), GEN, str(LMAX)])
    table = os.path.join(GEN, "boys_table.h")
    gen_src = os.path.join(CSRC, "boys_table_gen.c")
    exe = os.path.join(BUILD, "boys_table_gen")
    if not os.path.exists(table) or os.path.getmtime(table) < os.path.getmtime(gen_src):
        _run(["gcc", "-O2", "-o", exe, gen_src, "-lm"])
        _run([exe, table])
    units = []
    built = list(classes())
    lst = "// written by build.py\n#pragma once\n#define GS_FOR_EACH_BUILT(X) " + " ".join(
        "X(%d, %d, %d, %d)" % c for c in built) + "\n"
    path = os.path.join(GEN, "gs_built_classes.h")
    if not os.path.exists(path) or open(path).read() != lst:
        with open(path, "w") as f:
            f.write(lst)
    for cls in built:
        tag = "".join(map(str, cls))
        path = os.path.join(GEN, f"eri_k_{tag}.cu")
        L = sum(cls)
        if L < WIDE_PROG_MIN:
            # no warp program: the warp kernels are never selected below WIDE_PROG_MIN
            stub = ('// written by build.py -- no warp program below total angular momentum %d\n'
                    '#pragma once\nnamespace gs { template <> struct WideProg<%d, %d, %d, %d> '
                    '{ static constexpr int NVSLOT = 1, NVSEG = 0, VGROUP = 1, HSIZE = 1, NHLEV = 0; '
                    'static constexpr int NVSLOT_G = 1, NVSEG_G = 0; '
                    'static __device__ const uint4* vrec() { return nullptr; } '
                    'static __device__ const int* vseg() { return nullptr; } '
                    'static __device__ const unsigned short* vtgt() { return nullptr; } '
                    'static __device__ const uint4* vrec_g() { return nullptr; } '
                    'static __device__ const int* vseg_g() { return nullptr; } '
                    'static __device__ const unsigned short* vtgt_g() { return nullptr; } '
                    'static __device__ const unsigned int* hop() { return nullptr; } '
                    'static __device__ const int* hlev() { return nullptr; } '
                    'static __device__ const unsigned short* outslot() { return nullptr; } }; }\n'
                    % (WIDE_PROG_MIN, *cls))
            spath = os.path.join(GEN, f"eri_wide_{tag}.h")
            if not os.path.exists(spath) or open(spath).read() != stub:
                with open(spath, "w") as f:
                    f.write(stub)
        inc = '#include "eri_class_%s.h"\n#include "eri_wide_%s.h"\n' % (tag, tag)
        # GS_BOYS_ORDER: the Boys order of this class's kernels, whose Taylor rows the unit
        # embeds (eri_common.cuh)
        code = ('#define GS_BOYS_ORDER %d\n' % L +
                '#define GS_WIDE64_MIN %d\n#define GS_WIDE32_MIN %d\n#define GS_THREAD64_MAX %d\n'
                '#define GS_THREAD32_MAX %d\n#define GS_WIDE_FROM %d\n#define GS_WIDE32_FROM %d\n'
                '#include "eri_launch.cuh"\n%s'
                'int gs_launch_%s(int kind, int prec, const void* args, cudaStream_t st) {\n'
                '    return gs::launch_any<%d, %d, %d, %d>(kind, prec, args, st);\n}\n'
                'int gs_variants_%s(int prec) { return gs::variants<%d, %d, %d, %d>(prec); }\n'
                % (max(WIDE64_MIN, WIDE_PROG_MIN), max(WIDE32_MIN, WIDE_PROG_MIN), THREAD64_MAX,
                   THREAD32_MAX, WIDE_PROG_MIN, max(WIDE32_FROM, WIDE_PROG_MIN), inc, tag, *cls,
                   tag, *cls))
        if not os.path.exists(path) or open(path).read() != code:
            with open(path, "w") as f:
                f.write(code)
        deps = [os.path.join(GEN, f"eri_class_{tag}.h"), os.path.join(GEN, f"eri_wide_{tag}.h")]
        units.append((path, deps))
    # every class's recursion and warp program in one header, for the persistent kernels
    agg = "// written by build.py\n#pragma once\n" + "".join(
        '#include "eri_class_%s.h"\n#include "eri_wide_%s.h"\n' % (("".join(map(str, c)),) * 2)
        for c in built)
    path = os.path.join(GEN, "eri_all_classes.h")
    if not os.path.exists(path) or open(path).read() != agg:
        with open(path, "w") as f:
            f.write(agg)
    all_deps = [os.path.join(GEN, f"eri_{k}_{''.join(map(str, c))}.h") for c in built
                for k in ("class", "wide")] + [path, os.path.join(CSRC, "persistent.cuh")]
    for prec in (64, 32):
        units.append((os.path.join(CSRC, f"persistent{prec}.cu"), all_deps))
    # one translation unit per gradient class (the fused adjoint kernels, csrc/eri_grad.cuh)
    for cls in built:
        tag = "".join(map(str, cls))
        thread = sum(cls) <= GRAD_THREAD_LMAX
        inc = '#include "eri_grad_%s.h"\n' % tag + ('#include "eri_gradt_%s.h"\n' % tag if thread else "")
        # form: 1 thread per quartet, 2 warp per quartet, 3 split (the thread code, one warp
        # per quartet); the C entry checks that the thread forms exist for the class
        body = ('    if (form == 1) return gs::launch_grad_thread<%d, %d, %d, %d>(a, st);\n'
                '    if (form == 3) return gs::launch_grad_split<%d, %d, %d, %d>(a, st);\n'
                % (cls + cls) if thread else '    (void)form;\n')
        # the derivative integrals raise one centre: Boys order L + 1
        code = ('#define GS_BOYS_ORDER %d\n#include "eri_grad.cuh"\n%s'
                'int gs_grad_launch_%s(const gs::GradArgs& a, int form, cudaStream_t st) {\n%s'
                '    return gs::launch_grad<%d, %d, %d, %d>(a, st);\n}\n'
                % (sum(cls) + 1, inc, tag, body, *cls))
        path = os.path.join(GEN, f"eri_grad_k_{tag}.cu")
        if not os.path.exists(path) or open(path).read() != code:
            with open(path, "w") as f:
                f.write(code)
        deps = [os.path.join(CSRC, "eri_grad.cuh"), os.path.join(GEN, f"eri_grad_{tag}.h")]
        if thread:
            deps.append(os.path.join(GEN, f"eri_gradt_{tag}.h"))
        units.append((path, deps))
    return units


def _compile(src, deps, obj):
    common = [os.path.join(CSRC, n) for n in ("eri_common.cuh", "eri_kernels.cuh", "eri_wide.cuh",
                                              "eri_launch.cuh", "gs_args.h")]
    common.append(os.path.join(GEN, "boys_table.h"))
    key = _digest([src] + deps + common, " ".join(NVFLAGS))
    stamp = obj + ".key"
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == key:
        return obj, False
    _run([NVCC] + NVFLAGS + ["-c", src, "-o", obj])
    with open(stamp, "w") as f:
        f.write(key)
    return obj, True


def build(jobs=None, verbose=False):
    units = generate()
    objs = []
    todo = [(src, deps, os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")) for src, deps in units]
    todo.append((os.path.join(CSRC, "capi.cu"), [os.path.join(GEN, "gs_built_classes.h")],
                 os.path.join(BUILD, "capi.o")))
    todo.append((os.path.join(CSRC, "one_electron.cu"), [], os.path.join(BUILD, "one_electron.o")))
    todo.append((os.path.join(CSRC, "grad.cu"), [], os.path.join(BUILD, "grad.o")))
    todo.append((os.path.join(CSRC, "transform.cu"), [], os.path.join(BUILD, "transform.o")))
    todo.append((os.path.join(CSRC, "xc.cu"), [], os.path.join(BUILD, "xc.o")))
    todo.append((os.path.join(CSRC, "symmetry.cu"), [], os.path.join(BUILD, "symmetry.o")))
    todo.append((os.path.join(CSRC, "dense.cu"), [], os.path.join(BUILD, "dense.o")))
    todo.append((os.path.join(CSRC, "persistent_capi.cu"), [os.path.join(CSRC, "persistent.cuh")],
                 os.path.join(BUILD, "persistent_capi.o")))
    todo.append((os.path.join(CSRC, "eri_grad.cu"),
                 [os.path.join(CSRC, "eri_grad.cuh"), os.path.join(GEN, "eri_grad_list.h")],
                 os.path.join(BUILD, "eri_grad.o")))
    jobs = jobs or max(1, os.cpu_count() or 1)
    changed = False
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(_compile, *t) for t in todo]
        for f in futs:
            obj, did = f.result()
            objs.append(obj)
            changed |= did
    if changed or not os.path.exists(LIB):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    return LIB


def build_hostcheck():
    """CPU build of the generated recursions (tests only)."""
    generate()
    src = os.path.join(CSRC, "hostcheck.cpp")
    deps = [src, os.path.join(CSRC, "eri_common.cuh"), os.path.join(GEN, "eri_classes.h")]
    key = _digest(deps + [os.path.join(GEN, f"eri_class_{''.join(map(str, c))}.h") for c in classes()])
    stamp = HOSTCHECK + ".key"
    if os.path.exists(HOSTCHECK) and os.path.exists(stamp) and open(stamp).read() == key:
        return HOSTCHECK
    tmp = HOSTCHECK + ".tmp%d" % os.getpid()
    _run(["g++", "-O1", "-std=c++17", "-fPIC", "-shared", "-I", CSRC, "-I", GEN, "-o", tmp, src])
    os.replace(tmp, HOSTCHECK)
    with open(stamp, "w") as f:
        f.write(key)
    return HOSTCHECK


def opcount():
    with open(os.path.join(GEN, "opcount.json")) as f:
        return json.load(f)


if __name__ == "__main__":
    print(build())

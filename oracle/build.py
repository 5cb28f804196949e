"""Build recipe for the CPU oracle (TEST INFRASTRUCTURE ONLY).

* ``build_oracle()`` compiles ``oracle/sf_oracle.c`` -- the plain-C
  restatement of the reference algorithms -- into ``oracle/liboracle.so``.
  It runs wherever the tests run (build host and GPU host).
* ``build_ref()`` compiles golden-vector adapters (``oracle/ref_src/*.cc``)
  against the reference's own headers where they lie, into
  ``oracle/_ref/``.  It needs the reference checkout and therefore only runs
  on the build host; ``tests/golden/gen_golden.py`` uses the result to write
  the committed fixtures.

The reference is compiled with its generic one-lane ``VectorizedArray``
(ISA macros undefined, empty ``x86intrin.h`` stand-in), so the reference's
lane-interleaved DG vectors coincide with the cell-major layout used here.
Four reference headers (``evaluation_dg_laplacian.h``,
``evaluation_dg_advect.h``, ``precomputed_dg_laplacian.h``,
``matrix_vector_kernel.h``) are copied into ``oracle/_ref/patched/`` and
patched at build time (PATCHES below); nothing of the reference is stored in
the repository.

``build_oracle_perf()`` compiles the same oracle source for timing (the CPU
baseline of ``bench.py``).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: SF_REFERENCE_ROOT, else a checkout named
# "reference" beside this repository
REF_ROOT = os.environ.get("SF_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
REF_INC = os.path.join(REF_ROOT, "legacy", "include")
REF_SRC = os.path.join(REF_ROOT, "legacy", "src")
OUT_REF = os.path.join(HERE, "_ref")

# (file, 1-based line, expected text, replacement)
PATCHES = [
    # periodic x-wrap neighbour: '+ dofs_per_cell' must be '* dofs_per_cell'
    ("evaluation_dg_laplacian.h", 270,
     "(ii - (n_cells[0] - 1) * n_lanes) + dofs_per_cell",
     "(ii - (n_cells[0] - 1) * n_lanes) * dofs_per_cell"),
    # final x sweep integrates with the forward shape matrix; use transpose
    ("evaluation_dg_laplacian.h", 482,
     "apply_1d_matvec_kernel<nn, 1, 0, true, false, VectorizedArray<Number>>",
     "apply_1d_matvec_kernel<nn, 1, 0, false, false, VectorizedArray<Number>>"),
    ("evaluation_dg_advect.h", 435,
     "(ii-(n_cells[0]-1)*n_lanes)+dofs_per_cell",
     "(ii-(n_cells[0]-1)*n_lanes)*dofs_per_cell"),
    ("precomputed_dg_laplacian.h", 142,
     "(ii-(n_cells[0]-1)*n_lanes)+dofs_per_cell",
     "(ii-(n_cells[0]-1)*n_lanes)*dofs_per_cell"),
    # neighbour couplings of the precomputed SIPG matrices: the face-point
    # values are taken at the swapped ends (phi_0 at 1, phi_{N-1} at 0), which
    # are zero for the Hermite-like basis; the SIPG coupling of test phi_0(0)
    # with the left neighbour's phi_j(1) is
    # -tau phi_0(0) phi_j(1) - 1/2 phi_0'(0) phi_j(1) + 1/2 phi_j'(1) phi_0(0)
    ("precomputed_dg_laplacian.h", 344, "basis.value(0, 1.)*basis.value(N-1, 0.)",
     "basis.value(0, 0.)*basis.value(N-1, 1.)"),
    ("precomputed_dg_laplacian.h", 345, "+", "-"),
    ("precomputed_dg_laplacian.h", 346, "basis.derivative(0, 1.)*basis.value(N-1, 0.)",
     "basis.derivative(0, 0.)*basis.value(N-1, 1.)"),
    ("precomputed_dg_laplacian.h", 347, "-", "+"),
    ("precomputed_dg_laplacian.h", 348, "basis.derivative(N-1, 0.)*basis.value(0, 1.)",
     "basis.derivative(N-1, 1.)*basis.value(0, 0.)"),
    ("precomputed_dg_laplacian.h", 349, "basis.value(0, 1.)*basis.value(N-2, 0.)",
     "basis.value(0, 0.)*basis.value(N-2, 1.)"),
    ("precomputed_dg_laplacian.h", 350, "+", "-"),
    ("precomputed_dg_laplacian.h", 351, "basis.derivative(0, 1.)*basis.value(N-2, 0.)",
     "basis.derivative(0, 0.)*basis.value(N-2, 1.)"),
    ("precomputed_dg_laplacian.h", 352, "-", "+"),
    ("precomputed_dg_laplacian.h", 353, "basis.derivative(N-2, 0.)*basis.value(0, 1.)",
     "basis.derivative(N-2, 1.)*basis.value(0, 0.)"),
    # odd n, add_into, stride != 1: the middle entry of the summand must be
    # read at mid * stride (as the transposed branch at :159 does); only the
    # precomputed Laplacian's y mass product takes this branch
    ("matrix_vector_kernel.h", 86, "array_for_add[mid] +", "array_for_add[mid * stride] +"),
]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_oracle(force: bool = False) -> str:
    out = os.path.join(HERE, "liboracle.so")
    src = os.path.join(HERE, "sf_oracle.c")
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "sf_oracle.h"))):
        return out
    tmp = out + ".tmp%d" % os.getpid()
    _run(["gcc", "-O2", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-o", tmp, src, "-lm"])
    os.replace(tmp, out)
    return out


PERF_FLAGS = ["-O3", "-ffp-contract=fast", "-std=gnu11", "-fopenmp"]


def perf_target() -> list[str]:
    """CPU target of the timing build.  Arm hosts: -mcpu=native, the
    extensions the host reports (the named target -mcpu=neoverse-v2 enables
    extensions that the Grace hosts here do not expose, and its build died
    with SIGILL); other hosts: generic code.  The timed build is the CPU
    baseline only; the oracle build that results are checked against uses
    no CPU-specific flags."""
    import platform
    return ["-mcpu=native"] if platform.machine() in ("aarch64", "arm64") else []


def perf_build_flags() -> str:
    """the gcc flags liboracle_perf.so was built with (written beside it)"""
    path = os.path.join(HERE, "liboracle_perf.flags")
    return open(path).read().strip() if os.path.exists(path) else "unknown"


def build_oracle_perf(force: bool = False) -> str:
    """the oracle source compiled for timing as the CPU baseline: -O3, tuned
    for the host CPU on Arm hosts (perf_target), floating-point contraction
    allowed (the flags the reference's drivers are benchmarked with), OpenMP"""
    out = os.path.join(HERE, "liboracle_perf.so")
    flags_file = os.path.join(HERE, "liboracle_perf.flags")
    src = os.path.join(HERE, "sf_oracle.c")
    if not force and os.path.exists(out) and os.path.exists(flags_file) and os.path.getmtime(out) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "sf_oracle.h"))):
        return out
    tmp = out + ".tmp%d" % os.getpid()
    flags = PERF_FLAGS + perf_target()
    try:
        _run(["gcc"] + flags + ["-fPIC", "-shared", "-o", tmp, src, "-lm"])
    except RuntimeError:
        if flags == PERF_FLAGS:
            raise
        flags = list(PERF_FLAGS)  # the compiler does not know the target: generic code
        _run(["gcc"] + flags + ["-fPIC", "-shared", "-o", tmp, src, "-lm"])
    os.replace(tmp, out)
    with open(flags_file, "w") as f:
        f.write(" ".join(flags) + "\n")
    return out


def _patch_headers() -> str:
    pdir = os.path.join(OUT_REF, "patched")
    os.makedirs(pdir, exist_ok=True)
    by_file = {}
    for fname, line, old, new in PATCHES:
        by_file.setdefault(fname, []).append((line, old, new))
    for fname, edits in by_file.items():
        with open(os.path.join(REF_INC, fname)) as f:
            lines = f.readlines()
        for line, old, new in edits:
            if old not in lines[line - 1]:
                raise RuntimeError("reference %s:%d does not contain %r" % (fname, line, old))
            lines[line - 1] = lines[line - 1].replace(old, new)
        path, text = os.path.join(pdir, fname), "".join(lines)
        # rewritten only when the text changes, so that the adapters built on
        # it stay up to date
        if not os.path.exists(path) or open(path).read() != text:
            with open(path, "w") as f:
                f.write(text)
    return pdir


def build_ref() -> list[str]:
    """Compile the golden-vector adapters against the reference headers."""
    if not os.path.isdir(REF_INC):
        raise FileNotFoundError("reference checkout not found at %s" % REF_ROOT)
    os.makedirs(OUT_REF, exist_ok=True)
    pdir = _patch_headers()
    shim = os.path.join(HERE, "ref_src")
    flags = ["g++", "-O2", "-std=c++14", "-fPIC", "-shared", "-w",
             "-U__SSE2__", "-U__SSE__", "-U__AVX__", "-U__AVX2__", "-U__AVX512F__",
             "-I", shim]
    jobs = []
    # the DG headers put an OpenMP 'private' clause that the access macro of
    # ref_shim.h would rewrite, so they are built without OpenMP (serial)
    # the cell Laplacian's mass-matrix, convection and face variants are the
    # same adapter compiled with the reference's DO_MASS_MATRIX /
    # DO_CONVECTION / DO_FACES
    for name, src, extra, omp, defs in [("ref_kernel", "ref_kernel", [REF_INC], False, []),
                                        ("ref_cell_gll", "ref_cell_gll", [REF_INC, REF_SRC], True, []),
                                        ("ref_cell_hermite", "ref_cell_hermite", [REF_INC], False, []),
                                        ("ref_cell_mass", "ref_cell_hermite", [REF_INC], False,
                                         ["-DDO_MASS_MATRIX"]),
                                        ("ref_cell_convection", "ref_cell_hermite", [REF_INC], False,
                                         ["-DDO_CONVECTION"]),
                                        ("ref_cell_faces", "ref_cell_hermite", [REF_INC], False,
                                         ["-DDO_FACES"]),
                                        ("ref_cell_faces_convection", "ref_cell_hermite", [REF_INC], False,
                                         ["-DDO_FACES", "-DDO_CONVECTION"]),
                                        ("ref_dg", "ref_dg", [pdir, REF_INC], False, [])]:
        inc = ["-fopenmp"] if omp else []
        for d in extra:
            inc += ["-I", d]
        out = os.path.join(OUT_REF, "lib%s.so" % name)
        source = os.path.join(shim, src + ".cc")
        # inputs: the adapter, the shim headers, the included reference (and
        # patched) headers and this recipe
        deps = [source, os.path.abspath(__file__)] + glob.glob(os.path.join(shim, "*.h"))
        for d in extra:
            deps += glob.glob(os.path.join(d, "*.h"))
        jobs.append((out, flags + inc + defs + ["-o", out + ".tmp", source], deps))

    def one(job):
        out, cmd, deps = job
        if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps):
            return out
        _run(cmd)
        os.replace(out + ".tmp", out)
        return out

    with cf.ThreadPoolExecutor(min(len(jobs), os.cpu_count() or 1)) as ex:
        return list(ex.map(one, jobs))


if __name__ == "__main__":
    print(build_oracle(force=True))
    if len(sys.argv) > 1 and sys.argv[1] == "ref":
        for o in build_ref():
            print(o)

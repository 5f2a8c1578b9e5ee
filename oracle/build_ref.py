"""Build recipe for ``oracle/_ref``: the reference's own contact and integrator kernels, compiled
for the host CPU.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this file; only ``tests/``,
``__graft_entry__.build()/smoke()`` and ``bench.py``'s CPU reference arm use it.

The reference ships its two kernels as Jinja templates (``LIBRARIES/gpu_fine_contact_detection.cu``
and ``LIBRARIES/gpu_Verlet.cu``) and renders them with the physics constants baked in as literals
(``LIBRARIES/gpu_fine_contact_detection.py:10-15,92-103``, ``LIBRARIES/gpu_Verlet.py:10-15,63-73``).
This recipe does the same rendering, prepends a small host shim (``__device__``/``__global__``
erased, ``float3``/``double3`` structs, a serial or OpenMP-atomic ``atomicAdd``, thread-local
``blockIdx``/``threadIdx``) and appends an ``extern "C"`` driver that runs the kernel body once per
pair (or particle) with ``P`` = loop index.  Outputs go only to ``oracle/_ref/``, which git ignores.

Variants (``variant=``):
  ``"f32"``      the kernels as shipped (FP32 contact, FP64 Verlet);
  ``"f64"``      the contact kernel with every ``float`` turned into ``double``;
  ``"histfix"``  FP32 contact kernel with the tangential-history index ``displacement_tang[P+k]``
                 turned into ``displacement_tang[4*P+k]`` (the stride the arrays are allocated with).

The reference checkout is read from ``$MWDEM_REFERENCE_ROOT`` (else ``DEFAULT_REFERENCE_ROOT``, where the
checkout sits on the build machine) when it exists.  The rendered ``.cpp`` files
are kept next to the ``.so`` so that a machine without the reference checkout can still compile the
same renderings: ``ensure_built`` falls back to compiling an existing
rendered file.  Compiled with ``-ffp-contract=off`` because GCC on aarch64 fuses multiply-adds by
default, which would change FP32 rounding relative to the CUDA build (``--fmad=false``).
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
# the reference checkout on the machine that renders the templates (the GPU machine has none: it
# compiles the renderings carried along in _ref/)
DEFAULT_REFERENCE_ROOT = "/root/reference"
REFERENCE_ROOT = Path(os.environ.get("MWDEM_REFERENCE_ROOT") or DEFAULT_REFERENCE_ROOT)
CONTACT_TEMPLATE = REFERENCE_ROOT / "LIBRARIES" / "gpu_fine_contact_detection.cu"
VERLET_TEMPLATE = REFERENCE_ROOT / "LIBRARIES" / "gpu_Verlet.cu"

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
            "-fno-fast-math", "-w"]

_SHIM_COMMON = r"""
#include <cmath>
#include <cstdio>
#include <algorithm>
using std::min; using std::max; using std::sqrt; using std::log; using std::abs;
using std::sin; using std::cos;
#define __device__
#define __global__
struct mwd_dim3 { int x, y, z; };
static thread_local mwd_dim3 blockIdx, threadIdx;
static thread_local mwd_dim3 gridDim, blockDim;
static int mwd_parallel = 0;
"""

_SHIM_FLOAT3 = r"""
struct float3 { float x, y, z; };
static inline float3 make_float3(float x, float y, float z) { float3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline float atomicAdd(float* a, float v) {
    float old;
    if (mwd_parallel) {
        #pragma omp atomic capture
        { old = *a; *a += v; }
    } else { old = *a; *a = old + v; }
    return old;
}
"""

_SHIM_DOUBLE3 = r"""
struct double3 { double x, y, z; };
static inline double3 make_double3(double x, double y, double z) { double3 r; r.x = x; r.y = y; r.z = z; return r; }
"""


def _fmt(v):
    """Render a value the way the reference's Jinja call does (Python ``str`` of a float)."""
    return str(v)


def _contact_driver(real: str, V: int) -> str:
    return f"""
extern "C" void ref_contact_run(int n, int nthreads, int snapshot,
    {real}* Acom, {real}* Bcom, {real}* Av, {real}* Bv, {real}* Avel, {real}* Bvel,
    {real}* Aw, {real}* Bw, int* Anv, int* Bnv, int* Aid, int* Bid, {real}* hist,
    {real}* force, {real}* torque, {real}* qA, {real}* qB, int* pair_ids, int* collision,
    {real}* IsA, {real}* IsB, {real}* scratch)
{{
    /* snapshot != 0: every pair reads hist[P..P+2] as it was on entry and its four writes are
       recorded in scratch[4P..4P+3] (scratch[4P+3] stays NaN when the pair wrote nothing); the
       writes are then applied in pair order.  scratch must hold 4n values. */
    int np = n;
    auto body = [&](int P) {{
        {real}* hp = hist;
        if (snapshot) {{
            {real}* t = scratch + 4 * (size_t)P;
            t[0] = hist[P]; t[1] = hist[P + 1]; t[2] = hist[P + 2]; t[3] = NAN;
            hp = ({real}*)((char*)t - sizeof({real}) * (size_t)P);
        }}
        gridDim.x = 1; gridDim.y = 1; gridDim.z = 1;
        blockDim.x = 1; blockDim.y = 1; blockDim.z = 1;
        blockIdx.x = 0; blockIdx.y = P; blockIdx.z = 0;
        threadIdx.x = 0; threadIdx.y = 0; threadIdx.z = 0;
        contact_detection(({real}(*)[3])Acom, ({real}(*)[3])Bcom,
                          ({real}(*)[{V}][3])Av, ({real}(*)[{V}][3])Bv,
                          ({real}(*)[3])Avel, ({real}(*)[3])Bvel,
                          ({real}(*)[3])Aw, ({real}(*)[3])Bw,
                          Anv, Bnv, Aid, Bid, hp, force, torque,
                          ({real}(*)[4])qA, ({real}(*)[4])qB, &np, pair_ids, collision, IsA, IsB);
    }};
    if (nthreads <= 1) {{
        mwd_parallel = 0;
        for (int P = 0; P < n; ++P) body(P);
    }} else {{
        mwd_parallel = 1;
        #pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
        for (int P = 0; P < n; ++P) body(P);
        mwd_parallel = 0;
    }}
    if (snapshot) {{
        for (int P = 0; P < n; ++P) {{
            {real}* t = scratch + 4 * (size_t)P;
            if (t[3] == t[3]) {{ hist[P] = t[0]; hist[P + 1] = t[1]; hist[P + 2] = t[2]; hist[P + 3] = t[3]; }}
        }}
    }}
}}
"""


def _verlet_driver(N: int) -> str:
    return f"""
extern "C" void ref_verlet_run(int n, int nthreads,
    double* v, double* v12, double* w12bf, double* q12, double* q, double* qall,
    double* wbf, double* w, double* F, double* T, double* verts, double* com,
    double* mass, double* Iinv, double* I, double* dxall)
{{
    int np = n;
    auto body = [&](int P) {{
        gridDim.x = 1; gridDim.y = 1; gridDim.z = 1;
        blockDim.x = 1; blockDim.y = 1; blockDim.z = 1;
        blockIdx.x = 0; blockIdx.y = P; blockIdx.z = 0;
        threadIdx.x = 0; threadIdx.y = 0; threadIdx.z = 0;
        Verlet(v, v12, w12bf, q12, q, qall, wbf, w, (double(*)[3])F, (double(*)[3])T, verts, com,
               mass, (double(*)[3][3])Iinv, (double(*)[3][3])I, dxall, &np);
    }};
    if (nthreads <= 1) {{
        for (int P = 0; P < n; ++P) body(P);
    }} else {{
        #pragma omp parallel for num_threads(nthreads) schedule(static)
        for (int P = 0; P < n; ++P) body(P);
    }}
}}
"""


def render_contact(params: dict, variant: str = "f32") -> str:
    """Render the contact template exactly as ``gpu_contact_detection_init`` does, plus shim/driver.

    ``params`` keys follow ``gpu_fine_contact_detection.py:92-103``: Kn, en, et, Kn_wall, en_wall,
    et_wall, mu, mu_wall, num_vertices_max, num_particles_wall, timestep.
    """
    from jinja2 import Template
    src = CONTACT_TEMPLATE.read_text()
    args = {k: _fmt(params[k]) for k in ("Kn", "en", "et", "Kn_wall", "en_wall", "et_wall", "mu",
                                          "mu_wall", "timestep")}
    args["num_pairs"] = "1"
    args["num_vertices_max"] = str(int(params["num_vertices_max"]))
    args["num_particles_wall"] = str(int(params["num_particles_wall"]))
    body = Template(src).render(**args)
    if variant == "histfix":
        body = re.sub(r"displacement_tang\[P(\+\d)?\]", lambda m: "displacement_tang[4*P%s]" % (m.group(1) or ""), body)
    real = "float"
    head = _SHIM_COMMON
    if variant == "f64":
        head += "#define float double\n"
        real = "double"
    head += _SHIM_FLOAT3
    return head + body + _contact_driver(real, int(params["num_vertices_max"]))


def render_verlet(params: dict) -> str:
    """Render the integrator template exactly as ``gpu_Verlet_init`` does (``gpu_Verlet.py:63-73``)."""
    from jinja2 import Template
    src = VERLET_TEMPLATE.read_text()
    args = {k: _fmt(params[k]) for k in ("timestep_size", "syssize_x_max", "syssize_x_min",
                                          "syssize_y_max", "syssize_y_min", "syssize_z_max",
                                          "syssize_z_min")}
    for k in ("num_particles", "num_vertices_max", "num_part_min", "num_part_max"):
        args[k] = str(int(params[k]))
    body = Template(src).render(**args)
    # the reference prints on every fly-away reset; keep the print but make it line-buffered-safe
    return _SHIM_COMMON + _SHIM_DOUBLE3 + body + _verlet_driver(int(params["num_particles"]))


def _key(kind: str, params: dict, variant: str) -> str:
    blob = json.dumps({"kind": kind, "variant": variant, "params": {k: _fmt(v) for k, v in sorted(params.items())}},
                      sort_keys=True)
    return hashlib.sha1(blob.encode()).hexdigest()[:16]


def set_reference_root(path) -> None:
    """Read the reference templates from the checkout at `path` instead."""
    global REFERENCE_ROOT, CONTACT_TEMPLATE, VERLET_TEMPLATE
    REFERENCE_ROOT = Path(path)
    CONTACT_TEMPLATE = REFERENCE_ROOT / "LIBRARIES" / "gpu_fine_contact_detection.cu"
    VERLET_TEMPLATE = REFERENCE_ROOT / "LIBRARIES" / "gpu_Verlet.cu"


def reference_available() -> bool:
    return CONTACT_TEMPLATE.exists() and VERLET_TEMPLATE.exists()


def ensure_built(kind: str, params: dict, variant: str = "f32") -> Path:
    """Return the path of a compiled reference kernel library for ``params``; build it if needed.

    Raises ``FileNotFoundError`` when neither the reference templates nor a previously rendered
    source for these parameters exist (e.g. on a machine without the reference checkout).
    """
    REF_DIR.mkdir(parents=True, exist_ok=True)
    key = _key(kind, params, variant)
    cpp = REF_DIR / f"{kind}_{variant}_{key}.cpp"
    so = REF_DIR / f"{kind}_{variant}_{key}.so"
    if so.exists() and cpp.exists() and so.stat().st_mtime >= cpp.stat().st_mtime:
        return so
    if not cpp.exists():
        if not reference_available():
            raise FileNotFoundError(f"reference templates not found under {REFERENCE_ROOT} and no "
                                    f"pre-rendered source {cpp.name}")
        text = render_contact(params, variant) if kind == "contact" else render_verlet(params)
        cpp.write_text(text)
    tmp = so.with_suffix(".so.tmp%d" % os.getpid())
    subprocess.run(["g++", *CXXFLAGS, str(cpp), "-o", str(tmp)], check=True)
    os.replace(tmp, so)
    return so


def build_all_rendered() -> list:
    """Compile every rendered source already present in ``oracle/_ref`` (used on machines without
    the reference checkout, where only the rendered sources travel)."""
    out = []
    if not REF_DIR.exists():
        return out
    for cpp in sorted(REF_DIR.glob("*.cpp")):
        so = cpp.with_suffix(".so")
        if so.exists() and so.stat().st_mtime >= cpp.stat().st_mtime:
            out.append(so)
            continue
        tmp = so.with_suffix(".so.tmp%d" % os.getpid())
        subprocess.run(["g++", *CXXFLAGS, str(cpp), "-o", str(tmp)], check=True)
        os.replace(tmp, so)
        out.append(so)
    return out


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--rendered":
        for p in build_all_rendered():
            print(p)
    else:
        demo = dict(Kn=1e4, en=0.8, et=0.6, Kn_wall=1e2, en_wall=0.7, et_wall=0.6, mu=0.1, mu_wall=0.1,
                    num_vertices_max=8, num_particles_wall=0, timestep=1e-5)
        print(ensure_built("contact", demo))

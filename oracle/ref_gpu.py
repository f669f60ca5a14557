"""Recipe: the reference's own generated kernels, compiled for the GPU.

TEST/BASELINE INFRASTRUCTURE ONLY (the benchmark's same-GPU comparator; never
the product).

The reference compiles the CUDA C its translator generates with PyCUDA's
``SourceModule(source, options=["-w"])`` (``xentica/core/base.py:538-541``)
and launches ``emit`` then ``absorb`` once per ``step()``
(``base.py:703-728``) with the block and grid PyCUDA's ``gpuarray.splay``
picks for the cell array.  This recipe takes the same translator output --
the LifelikeCA sources ``ref_build.py`` dumps into ``oracle/_ref`` for every
lattice size of the ensemble benchmark -- puts each size's kernels in a
namespace of one ``.cu`` file, adds a C launcher that replays that calling
pattern (one emit and one absorb launch per lattice per generation, from a
C loop rather than Python, so launch overhead is the CUDA runtime's alone),
and compiles it with nvcc for sm_103a into ``oracle/_ref/libref_gpu.so``.
PyCUDA itself is not needed and not installed.
"""
import glob
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
CU = os.path.join(REF_DIR, "ref_lifelike_gpu.cu")
LIB = os.path.join(REF_DIR, "libref_gpu.so")

# the generated source ends where ref_harness.py appended its CPU wrappers
_WRAPPER_MARK = "#include <omp.h>"

_RUNNER = r'''
typedef void (*xkrefg_emit_t)(unsigned char *, int);
typedef void (*xkrefg_absorb_t)(unsigned char *, int3 *, int, int);
struct XkrefgEntry { int w, h; xkrefg_emit_t emit; xkrefg_absorb_t absorb; };
static const XkrefgEntry kXkrefg[] = {
%(table)s
};
static const int kXkrefgCount = %(count)d;

// PyCUDA's gpuarray.splay (block and grid of an n-element array): warp-sized
// blocks up to 4 blocks per SM, then wider blocks up to 128 threads
static void xkrefg_splay(long long n, int sms, int *blocks, int *threads)
{
    const long long min_threads = 32, max_threads = 128, max_blocks = 4LL * sms;
    if (n < min_threads) { *blocks = 1; *threads = (int)min_threads; }
    else if (n < max_blocks * min_threads) {
        *blocks = (int)((n + min_threads - 1) / min_threads);
        *threads = (int)min_threads;
    } else if (n < max_blocks * max_threads) {
        *blocks = (int)max_blocks;
        const long long grp = (n + min_threads - 1) / min_threads;
        *threads = (int)(((grp + max_blocks - 1) / max_blocks) * min_threads);
    } else { *blocks = (int)max_blocks; *threads = (int)max_threads; }
}

struct XkrefgLattice { int entry, n, rule, blocks, threads; unsigned char *fld; int3 *col; };
struct XkrefgRun { int count; XkrefgLattice *lat; cudaEvent_t e0, e1; };

extern "C" void xkrefg_destroy(XkrefgRun *r)
{
    if (!r) return;
    for (int i = 0; i < r->count; ++i) {
        if (r->lat[i].fld) cudaFree(r->lat[i].fld);
        if (r->lat[i].col) cudaFree(r->lat[i].col);
    }
    if (r->e0) cudaEventDestroy(r->e0);
    if (r->e1) cudaEventDestroy(r->e1);
    delete[] r->lat;
    delete r;
}

// lattices of the given sizes and rules; cells: their main planes (one byte
// per cell) concatenated.  Returns null if a size has no generated kernels
// or CUDA fails.
extern "C" XkrefgRun *xkrefg_create(int count, const int *w, const int *h, const int *rule,
                                    const unsigned char *cells)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return nullptr;
    XkrefgRun *r = new XkrefgRun();
    r->count = count;
    r->lat = new XkrefgLattice[count]();
    cudaEventCreate(&r->e0);
    cudaEventCreate(&r->e1);
    long long off = 0;
    for (int i = 0; i < count; ++i) {
        XkrefgLattice &L = r->lat[i];
        L.entry = -1;
        for (int k = 0; k < kXkrefgCount; ++k)
            if (kXkrefg[k].w == w[i] && kXkrefg[k].h == h[i]) L.entry = k;
        L.n = w[i] * h[i];
        L.rule = rule[i];
        const long long planes = 9LL * L.n + 1;      // main + 8 buffers + 1 (base.py:553-557)
        xkrefg_splay(planes, sms, &L.blocks, &L.threads);
        if (L.entry < 0 || cudaMalloc(&L.fld, planes) != cudaSuccess ||
            cudaMalloc(&L.col, sizeof(int3) * (size_t)L.n) != cudaSuccess ||
            cudaMemset(L.fld, 0, planes) != cudaSuccess ||
            cudaMemset(L.col, 0, sizeof(int3) * (size_t)L.n) != cudaSuccess ||
            cudaMemcpy(L.fld, cells + off, (size_t)L.n, cudaMemcpyHostToDevice) != cudaSuccess) {
            xkrefg_destroy(r);
            return nullptr;
        }
        off += L.n;
    }
    return r;
}

// `generations` steps of every lattice, generation-major like a host loop
// over models: emit then absorb per lattice; returns the device time in ms
// (negative on a CUDA error)
extern "C" float xkrefg_step(XkrefgRun *r, int generations)
{
    cudaEventRecord(r->e0, 0);
    for (int g = 0; g < generations; ++g)
        for (int i = 0; i < r->count; ++i) {
            const XkrefgLattice &L = r->lat[i];
            kXkrefg[L.entry].emit<<<L.blocks, L.threads>>>(L.fld, L.n);
            kXkrefg[L.entry].absorb<<<L.blocks, L.threads>>>(L.fld, L.col, L.rule, L.n);
        }
    cudaEventRecord(r->e1, 0);
    if (cudaEventSynchronize(r->e1) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return -1.f;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r->e0, r->e1);
    return ms;
}

extern "C" int xkrefg_download(XkrefgRun *r, unsigned char *cells)
{
    long long off = 0;
    for (int i = 0; i < r->count; ++i) {
        if (cudaMemcpy(cells + off, r->lat[i].fld, (size_t)r->lat[i].n, cudaMemcpyDeviceToHost) !=
            cudaSuccess)
            return -1;
        off += r->lat[i].n;
    }
    return 0;
}
'''


def _sources():
    out = []
    for cpp in sorted(glob.glob(os.path.join(REF_DIR, "ref_lifelike_*.cpp"))):
        m = re.search(r"ref_lifelike_(\d+)x(\d+)\.cpp$", cpp)
        with open(cpp) as fh:
            text = fh.read()
        if _WRAPPER_MARK not in text:
            continue
        out.append((int(m.group(1)), int(m.group(2)), text.split(_WRAPPER_MARK)[0]))
    return out


def generate():
    """Write ``ref_lifelike_gpu.cu``; returns its path, or None without sources."""
    srcs = _sources()
    if not srcs:
        return None
    parts = ["// Generated by oracle/ref_gpu.py from the reference translator's LifelikeCA\n"
             "// output (one namespace per lattice size).  Test infrastructure only.\n"
             "#include <cuda_runtime.h>\n"]
    table = []
    for w, h, src in srcs:
        ns = "xkref_%dx%d" % (w, h)
        macros = re.findall(r"^#define\s+(\w+)", src, flags=re.M)
        parts.append("namespace %s {\n%s\n}  // namespace %s\n" % (ns, src, ns))
        parts.append("".join("#undef %s\n" % mac for mac in macros))
        table.append("    {%d, %d, %s::emit, %s::absorb}," % (w, h, ns, ns))
    parts.append(_RUNNER % {"table": "\n".join(table), "count": len(table)})
    text = "\n".join(parts)
    if not os.path.exists(CU) or open(CU).read() != text:
        with open(CU, "w") as fh:
            fh.write(text)
    return CU


def nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else "nvcc"


def build():
    """Generate and compile (idempotent); returns the library path or None."""
    cu = generate()
    if cu is None:
        return None
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(cu):
        tmp = LIB + ".tmp"
        # -w as the reference passes to SourceModule; -O3 as nvcc's default
        cmd = [nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w", "-shared",
               "-Xcompiler", "-fPIC", cu, "-o", tmp, "-lcudart"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


def available():
    """Path of the compiled library, or None."""
    return LIB if os.path.exists(LIB) else None


if __name__ == "__main__":
    print(build())

"""Build recipe for the refrakt_gb300 shared library (sm_103a).

Compiles refrakt_gb300/csrc/*.cu and *.cpp with nvcc into refrakt_gb300/_lib/librefrakt_gb300.so
(in-tree, git-ignored).  Translation units compile in parallel; one -gencode target.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "librefrakt_gb300.so")
OBJ_DIR = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")


# device headers the run-time compiler sees (specialize.cpp), embedded into the library
RTC_HEADERS = ["rtc_types.h", "program.h", "device.cuh", "variations.cuh", "splat.cuh", "chaos_args.h",
               "chaos_body.cuh", "batch_args.h", "batch_body.cuh"]


def _rtc_headers_source():
    """Writes _build/rtc_headers.cpp: the RTC_HEADERS as string literals (kRtcHeader*)."""
    out = os.path.join(OBJ_DIR, "rtc_headers.cpp")
    parts = ["// generated by nvbuild.py: device headers for the run-time compiler", "namespace rfk {",
             "extern const int kRtcHeaderCount = %d;" % len(RTC_HEADERS),
             "extern const char* const kRtcHeaderNames[] = {%s};" % ", ".join('"%s"' % h for h in RTC_HEADERS),
             "extern const char* const kRtcHeaderSources[] = {"]
    for h in RTC_HEADERS:
        with open(os.path.join(CSRC, h)) as f:
            text = f.read()
        assert ")RFKHDR\"" not in text
        parts.append('R"RFKHDR(%s)RFKHDR",' % text)
    parts += ["};", "}  // namespace rfk", ""]
    body = "\n".join(parts)
    if not os.path.exists(out) or open(out).read() != body:
        with open(out, "w") as f:
            f.write(body)
    return out


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp"))) + \
        [_rtc_headers_source()]


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                  glob.glob(os.path.join(ROOT, "include", "*.h")))


def _flags():
    return ["-O3", "-std=c++17", "-lineinfo", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
            "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden"] + ARCH


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = _sources()
    newest_hdr = max(os.path.getmtime(h) for h in _headers())
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(OBJ_DIR, os.path.basename(s) + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), newest_hdr):
            jobs.append((s, o))

    def compile_one(job):
        s, o = job
        cmd = [NVCC] + _flags() + ["-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return s, r

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for s, r in ex.map(compile_one, jobs):
                if r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                    raise RuntimeError("nvcc failed on " + s)
                if verbose and (r.stdout or r.stderr):
                    sys.stderr.write(r.stdout + r.stderr)
    stale = not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs)
    if force or jobs or stale:
        tmp = LIB + ".tmp.%d" % os.getpid()
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

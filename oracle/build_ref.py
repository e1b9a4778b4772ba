"""Recipe that builds the reference NSW6 code as a test oracle (TEST INFRASTRUCTURE ONLY).

The reference (Masahiro-Ren/nicam_kokkos_microphysics) is C++17 written
against Kokkos >= 4.6.1, which is not installed.  This recipe

  1. copies the reference's sources (src/*.cpp except main.cpp, include/*.h)
     unmodified into the git-ignored output directory ``oracle/_ref/src``,
  2. writes, per problem size, a copy of the headers whose compile-time sizes
     in include/problemsize.h:62-79 (ADM_gall_in, ADM_kall, ADM_vlayer,
     ADM_kmax, kmax) are replaced by the requested ones,
  3. compiles those sources with g++ against our host-only Kokkos shim
     (``oracle/kokkos_shim``) together with ``oracle/ref_driver.cpp`` (which
     replaces main.cpp) into ``oracle/_ref/<variant>_g<gall>_k<kall>/libnsw6ref.so``.

Variants:
  strict  serial shim, -O2 -ffp-contract=off: the deterministic oracle.
  omp     OpenMP shim, -O3 -fopenmp: the reference's Kokkos-OpenMP CPU build.
  fma     contraction on: the reference's own build-to-build spread.
  opt     as strict, with the two scheme choices that mp_nsw6_init assigns from
          literals (Roh_flag = true, qr_aut_acc_type = "KK2000",
          src/mod_mp_nsw6.cpp:291-292) turned into variables the driver sets,
          so that the switches mp_nsw6_init and precip_transport_new read
          (Roh_flag, OPT_EXPLICIT_ICEGEN, qr_aut_acc_type, OPT_INDIR,
          precip_transport_type, PRCIP_TRN_ECORRECT) can all be flipped; with
          the defaults it computes exactly what strict computes.

The reference tree is found at ``--reference-root`` (or the environment
variable NSW6_REFERENCE_ROOT), else in a checkout named ``reference`` beside
this repository.  When it is absent (on a machine that only received the
repository), the copy already in ``oracle/_ref/src`` is used if present.
Everything written goes to ``oracle/_ref/`` only.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import platform
import re
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
# the reference checkout: NSW6_REFERENCE_ROOT, else "reference" beside this repository
REF_ROOT = Path(os.environ.get("NSW6_REFERENCE_ROOT") or HERE.parent.parent / "reference")
OUT = HERE / "_ref"
SRC_COPY = OUT / "src"
SHIM = HERE / "kokkos_shim"

# Translation units of the reference that the hot path needs (main.cpp is
# replaced by ref_driver.cpp).
REF_UNITS = [
    "problemsize.cpp",
    "data_io.cpp",
    "mod_debug.cpp",
    "mod_thrmdyn.cpp",
    "mod_satadjust.cpp",
    "mod_vadv1d.cpp",
    "mod_precip_transport.cpp",
    "mod_mp_nsw6.cpp",
    "mod_mp_driver.cpp",
]

VARIANT_FLAGS = {
    "strict": ["-O2", "-ffp-contract=off"],
    "omp": ["-O3", "-fopenmp", "-DNSW6_SHIM_OPENMP"],
    # fused multiply-add contraction, as the reference's GPU (nvcc) and -Ofast
    # builds compile it: measures the reference's own build-to-build spread
    "fma": ["-O2", "-ffp-contract=fast"] + (["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []),
    "opt": ["-O2", "-ffp-contract=off", "-DNSW6REF_OPTIONS"],
}

# The literal assignments of mp_nsw6_init that the "opt" variant replaces.
OPT_PATCHES = [
    ("    Roh_flag = true;\n", "    Roh_flag = nsw6ref_opt_roh;\n"),
    ('    qr_aut_acc_type = "KK2000";\n', '    qr_aut_acc_type = nsw6ref_opt_kk2000 ? "KK2000" : "Default";\n'),
]
OPT_DECL = "extern bool nsw6ref_opt_roh;\nextern bool nsw6ref_opt_kk2000;\n"


def patched_nsw6(text: str) -> str:
    for a, b in OPT_PATCHES:
        if text.count(a) != 1:
            raise RuntimeError(f"mod_mp_nsw6.cpp: expected one occurrence of {a.strip()!r}")
        text = text.replace(a, b)
    return OPT_DECL + text


def sources_available() -> bool:
    return (REF_ROOT / "src" / "mod_mp_nsw6.cpp").is_file() or (SRC_COPY / "src" / "mod_mp_nsw6.cpp").is_file()


def refresh_copy() -> Path:
    """Copy the reference sources into oracle/_ref/src (unmodified)."""
    if (REF_ROOT / "src" / "mod_mp_nsw6.cpp").is_file():
        for sub in ("src", "include"):
            dst = SRC_COPY / sub
            dst.mkdir(parents=True, exist_ok=True)
            for f in sorted((REF_ROOT / sub).iterdir()):
                if f.suffix in (".cpp", ".h") and f.name != "main.cpp":
                    tgt = dst / f.name
                    if not tgt.exists() or tgt.read_bytes() != f.read_bytes():
                        shutil.copyfile(f, tgt)
    if not (SRC_COPY / "src" / "mod_mp_nsw6.cpp").is_file():
        raise FileNotFoundError("reference sources not found (neither the reference tree nor oracle/_ref/src)")
    return SRC_COPY


def patched_problemsize(text: str, gall: int, kall: int) -> str:
    kmax = kall - 2

    def sub(name: str, value: int, s: str) -> str:
        pat = re.compile(r"(constexpr\s+size_t\s+" + name + r"\s*=\s*)\d+")
        s2, n = pat.subn(lambda m: m.group(1) + str(value), s, count=1)
        if n != 1:
            raise RuntimeError(f"problemsize.h: could not patch {name}")
        return s2

    text = sub("ADM_gall_in_orig", gall, text)
    text = sub("ADM_gall_in", gall, text)
    text = sub("ADM_kall", kall, text)
    text = sub("ADM_vlayer", kall - 2, text)
    text = sub("ADM_kmax", kmax, text)
    text = sub("kmax", kmax, text)
    return text


def lib_path(gall: int, kall: int, variant: str = "strict") -> Path:
    return OUT / f"{variant}_g{gall}_k{kall}" / "libnsw6ref.so"


def build(gall: int, kall: int, variant: str = "strict", jobs: int | None = None, force: bool = False) -> Path:
    src = refresh_copy()
    bdir = OUT / f"{variant}_g{gall}_k{kall}"
    inc = bdir / "include"
    inc.mkdir(parents=True, exist_ok=True)
    for h in sorted((src / "include").iterdir()):
        text = h.read_text()
        if h.name == "problemsize.h":
            text = patched_problemsize(text, gall, kall)
        tgt = inc / h.name
        if not tgt.exists() or tgt.read_text() != text:
            tgt.write_text(text)

    units = [src / "src" / u for u in REF_UNITS] + [HERE / "ref_driver.cpp"]
    if variant == "opt":
        psrc = bdir / "mod_mp_nsw6.cpp"
        text = patched_nsw6((src / "src" / "mod_mp_nsw6.cpp").read_text())
        if not psrc.exists() or psrc.read_text() != text:
            psrc.write_text(text)
        units = [psrc if u.name == "mod_mp_nsw6.cpp" else u for u in units]

    so = bdir / "libnsw6ref.so"
    deps = units + [SHIM / "Kokkos_Core.hpp", Path(__file__)]
    if so.exists() and not force and all(so.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return so

    flags = ["g++", "-std=c++17", "-fPIC", "-w", f"-I{inc}", f"-I{src / 'src'}", f"-I{SHIM}"] + VARIANT_FLAGS[variant]

    def compile_one(u: Path) -> Path:
        obj = bdir / (u.stem + ".o")
        subprocess.run(flags + ["-c", str(u), "-o", str(obj)], check=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(units), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, units))
    link = ["g++", "-shared", "-o", str(so)] + [str(o) for o in objs]
    if variant == "omp":
        link.append("-fopenmp")
    subprocess.run(link, check=True)
    for o in objs:
        o.unlink()
    return so


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gall", type=int, required=True)
    ap.add_argument("--kall", type=int, required=True)
    ap.add_argument("--variant", choices=sorted(VARIANT_FLAGS), default="strict")
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--reference-root", type=Path, default=None,
                    help="the reference checkout (default: NSW6_REFERENCE_ROOT, else ../reference)")
    a = ap.parse_args(argv)
    if a.reference_root is not None:
        global REF_ROOT
        REF_ROOT = a.reference_root
    print(build(a.gall, a.kall, a.variant, force=a.force))
    return 0


if __name__ == "__main__":
    sys.exit(main())

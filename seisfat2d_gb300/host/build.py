"""Build recipe of the C++ drop-in (Modeling/Eikonal/Geometry/admin,
Inversion/Tomography_ISO) and its drivers: modeling.exe, inversion.exe,
traveltime_tables.exe, all linked against libseisfat2d.so."""
import concurrent.futures as cf
import os
import subprocess

from .. import build as lib_build

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
LIBSRC = ["admin.cpp", "geometry.cpp", "modeling.cpp", "inversion.cpp"]
EXES = {"modeling.exe": "modeling_main.cpp", "inversion.exe": "inversion_main.cpp",
        "migration.exe": "migration_main.cpp",
        "traveltime_tables.exe": "tables_main.cpp"}
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-I", lib_build.INC,
         "-I", os.path.join(CUDA, "include")]


def exe_path(name):
    return os.path.join(OUT, name)


def build(force=False):
    lib = lib_build.build()
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith((".cpp", ".hpp"))]
    newest = max(os.path.getmtime(s) for s in srcs + [lib])
    if not force and all(os.path.exists(exe_path(e)) and os.path.getmtime(exe_path(e)) >= newest for e in EXES):
        return OUT

    def obj(src):
        o = os.path.join(OUT, src.replace(".cpp", ".o"))
        subprocess.run(["g++"] + FLAGS + ["-c", os.path.join(HERE, src), "-o", o], check=True)
        return o

    with cf.ThreadPoolExecutor(8) as ex:
        objs = list(ex.map(obj, LIBSRC + list(EXES.values())))
    common = objs[:len(LIBSRC)]
    libdir = os.path.dirname(lib)
    for k, (exe, main) in enumerate(EXES.items()):
        mo = objs[len(LIBSRC) + k]
        subprocess.run(["g++", "-o", exe_path(exe), mo] + common +
                       ["-L", libdir, "-lseisfat2d", "-Wl,-rpath," + libdir,
                        "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(CUDA, "lib64")],
                       check=True)
    return OUT


if __name__ == "__main__":
    print(build(force=True))

"""Build recipe and wrapper of the reference's own SDF reader (TEST
INFRASTRUCTURE: only tests/ use it, to check this package's SDF dumps).

The reference ships its SDF C library as plain C (SDF/C/src/*.c, header
SDF/C/include/sdf.h, vendored uthash).  Its build generates one header,
commit_info.h, holding two version strings (SDF/C/src/gen_commit_string.sh);
this recipe writes that header itself with "unknown" for both and compiles
the library's sources where they lie, with gcc, together with
oracle/sdf_ref_dump.c, into oracle/_ref/sdf_ref_dump.  Nothing of the
reference is copied into the repository.  Where the reference tree is absent
(the GPU machine), build() returns None and the tests that need it skip.
"""
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
EXE = os.path.join(REF, "sdf_ref_dump")
SDF_C = os.environ.get("CYL_REFERENCE_SDF_C", "/root/reference/SDF/C")


def build(force=False):
    """Compile the reference's SDF C library and the dump program; returns
    the program's path, or None when the reference's sources are absent."""
    srcs = sorted(glob.glob(os.path.join(SDF_C, "src", "*.c")))
    if not srcs:
        return EXE if os.path.exists(EXE) else None
    me = os.path.join(HERE, "sdf_ref_dump.c")
    if not force and os.path.exists(EXE) and os.path.getmtime(EXE) >= os.path.getmtime(me):
        return EXE
    stub = os.path.join(REF, "stub")
    os.makedirs(stub, exist_ok=True)
    with open(os.path.join(stub, "commit_info.h"), "w") as f:
        f.write('#define SDF_COMMIT_ID "unknown"\n#define SDF_COMMIT_DATE "unknown"\n')
    cmd = ["gcc", "-O1", "-std=gnu99", "-I", os.path.join(SDF_C, "include"), "-I", os.path.join(SDF_C, "src"),
           "-I", stub, "-o", EXE + ".tmp", me] + srcs + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference SDF reader build failed: {' '.join(cmd)}\n{r.stderr}")
    os.replace(EXE + ".tmp", EXE)
    return EXE


def read(path):
    """The file as the reference's reader sees it: (header dict, list of
    blocks), each block a dict with id, name, blocktype, datatype, dims,
    stagger, mesh_id, units and its data (a numpy array), grids (list of
    arrays) or constant."""
    import numpy as np
    exe = build()
    if exe is None:
        raise FileNotFoundError("the reference's SDF C library is not available")
    out = subprocess.run([exe, str(path)], capture_output=True, text=True, check=True).stdout
    header, blocks = None, []
    for line in out.splitlines():
        tag, _, rest = line.partition(" ")
        if tag == "HEADER":
            f = rest.split(" ", 4)
            header = {"step": int(f[0]), "time": float(f[1]), "nblocks": int(f[2]), "restart": int(f[3]),
                      "code_name": f[4] if len(f) > 4 else ""}
        elif tag == "BLOCK":
            f = rest.split("\t")
            blocks.append({"id": f[0], "name": f[1], "blocktype": int(f[2]), "datatype": int(f[3]),
                           "ndims": int(f[4]), "dims": [int(v) for v in f[5].split(",")] if f[5] else [],
                           "stagger": int(f[6]), "mesh_id": f[7], "units": f[8], "grids": []})
        elif tag == "CONST":
            blocks[-1]["constant"] = float(rest)
        elif tag == "DATA":
            v = rest.split()
            if blocks[-1]["datatype"] in (1, 2):  # integer4, integer8
                blocks[-1]["data"] = np.array([int(x) for x in v[1:]], dtype=np.int64)
            else:
                blocks[-1]["data"] = np.array([float(x) for x in v[1:]])
        elif tag == "GRID":
            v = rest.split()
            blocks[-1]["grids"].append(np.array([float(x) for x in v[2:]]))
        elif tag == "READ_ERROR":
            blocks[-1]["read_error"] = True
    return header, blocks

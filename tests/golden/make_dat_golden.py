"""Generate dat_golden.json: what the reference's own DatFile::parseDatFile (reader.cpp, compiled
unmodified into oracle/_ref by oracle/build_ref.sh) returns for each case of dat_cases.py.

    sh oracle/build_ref.sh && python tests/golden/make_dat_golden.py

Run from any directory; the cases are written to a temporary directory, and the parser runs
with an empty working directory so raw files resolve relative to the .dat file."""
import ctypes as C
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from dat_cases import CASES, make_case  # noqa: E402

REF = os.path.join(HERE, "..", "..", "oracle", "_ref", "libvvref_sobel.so")


def ref_parse(lib, path):
    raw = C.create_string_buffer(1024)
    sizes, dists = (C.c_int * 3)(), (C.c_float * 3)()
    t, dim, b, e = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    st = lib.vvref_dat_parse(path.encode(), raw, 1024, sizes, dists, C.byref(t), C.byref(dim), C.byref(b), C.byref(e))
    if st != 0:
        return {"ok": False}
    return {"ok": True, "raw_file": raw.value.decode(), "resolution": list(sizes), "slice_thickness": list(dists),
            "format": t.value, "components": dim.value, "timestep_begin": b.value, "timestep_end": e.value}


def main():
    lib = C.CDLL(os.path.abspath(REF))
    out = {}
    with tempfile.TemporaryDirectory() as root:
        cwd = os.path.join(root, "_cwd")
        os.makedirs(cwd)
        old = os.getcwd()
        os.chdir(cwd)
        try:
            for name, text, raws in CASES:
                p = make_case(root, name, text, raws)
                r = ref_parse(lib, p)
                if r["ok"]:
                    r["raw_file"] = r["raw_file"].replace(os.path.join(root, name), "<DIR>")
                out[name] = r
        finally:
            os.chdir(old)
    with open(os.path.join(HERE, "dat_golden.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print(f"wrote {len(out)} cases")


if __name__ == "__main__":
    main()

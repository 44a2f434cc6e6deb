"""The Fortran side of the boundary (fortran/dftbgpu.F90) against the C header, without a Fortran
compiler: the bind(C) derived types have the C structs' member order, kinds and offsets (gcc prints
offsetof/sizeof of include/dftbgpu.h), every bind(C) interface names an entry point the header
declares with the same number of arguments, and a C program that dlopens libdftbgpu.so can call
dftbgpu_create (on a machine without a GPU it reports DFTBGPU_ERR_NO_DEVICE)."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "dftbgpu.h")
F90 = os.path.join(ROOT, "fortran", "dftbgpu.F90")

C_KINDS = {"real(c_double)": ("double", 8), "integer(c_int)": ("int", 4)}


def _strip_comments(src):
    return "\n".join(line.split("!")[0] for line in src.splitlines())


def _fortran_types():
    src = _strip_comments(open(F90).read())
    out = {}
    for m in re.finditer(r"type\s*,\s*bind\(C\)\s*::\s*(\w+)(.*?)end type", src, re.S | re.I):
        fields = []
        for line in m.group(2).splitlines():
            fm = re.match(r"\s*(real\(c_double\)|integer\(c_int\))\s*::\s*(.+)", line, re.I)
            if fm:
                for name in fm.group(2).split(","):
                    fields.append((name.strip(), C_KINDS[fm.group(1).lower()]))
        out[m.group(1)] = fields
    return out


def _c_layout(fields):
    off, res, align = 0, [], 1
    for name, (ctype, size) in fields:
        off = (off + size - 1) // size * size
        res.append((name, off, size))
        off += size
        align = max(align, size)
    return res, (off + align - 1) // align * align


@pytest.fixture(scope="module")
def abi_exe(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    exe = str(tmp_path_factory.mktemp("abi") / "abi_layout")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_layout.c"), "-o", exe, "-ldl"], check=True)
    return exe


def test_bind_c_types_match_header(abi_exe):
    out = subprocess.run([abi_exe, "layout"], check=True, capture_output=True, text=True).stdout
    c_fields, c_size = {}, {}
    for line in out.splitlines():
        p = line.split()
        if p[1] == "sizeof":
            c_size[p[0]] = int(p[2])
        else:
            c_fields.setdefault(p[0], []).append((p[1], int(p[2]), int(p[3])))
    ftypes = _fortran_types()
    for fname, cname in (("TDftbGpuOpts", "dftbgpu_scc_opts"), ("TDftbGpuEnergies", "dftbgpu_energies")):
        layout, size = _c_layout(ftypes[fname])
        assert size == c_size[cname], (fname, size, c_size[cname])
        assert len(layout) == len(c_fields[cname]), fname
        for (fn, fo, fs), (cn, co, cs) in zip(layout, c_fields[cname]):
            assert (fo, fs) == (co, cs), (fname, fn, cn, fo, co, fs, cs)


def _header_arg_counts():
    src = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(?:int|void|long long|const char \*)\s*\**\s*(dftbgpu_\w+)\s*\(([^)]*)\)\s*;", src):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else len(args.split(","))
    return out


def test_fortran_interfaces_name_header_entry_points():
    hdr = _header_arg_counts()
    src = _strip_comments(open(F90).read()).replace("&\n", " ").replace("&", " ")
    found = 0
    for m in re.finditer(r"(?:function|subroutine)\s+(\w+)\s*\(([^)]*)\)[^\n]*?bind\(C,\s*name=\"(\w+)\"\)", src,
                         re.I):
        cname = m.group(3)
        nargs = len([a for a in m.group(2).split(",") if a.strip()])
        assert cname in hdr, cname
        assert hdr[cname] == nargs, (cname, hdr[cname], nargs)
        found += 1
    assert found >= 14


def test_c_program_loads_library(abi_exe):
    from dftbplus_gb300 import build
    lib = build.build()
    out = subprocess.run([abi_exe, "create", lib], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    rc = int(out.stdout.split()[-1])
    assert rc in (0, 8), out.stdout     # a context, or DFTBGPU_ERR_NO_DEVICE where there is no GPU

"""The Fortran binding (include/pfgpu_mod.F90) against the C header.

No Fortran compiler exists here, so the bind(C) types are checked the way a
compiler would lay them out: each type's members are parsed from the module
(names, order, interoperable kinds, fixed-size arrays), their C-interop
offsets computed from the kinds' sizes and natural alignment, and compared
with offsetof/sizeof of the same struct compiled by gcc from pfgpu.h.  A
member added to a struct in the header but not to the module (or in another
place, or with another kind) fails here.  The interfaces are checked against
the header's prototypes by name and argument count."""
import os
import re
import shutil
import subprocess
import tempfile

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "pfgpu.h")
MODULE = os.path.join(REPO, "include", "pfgpu_mod.F90")

# Fortran type <-> C struct
TYPES = {"pf_sorption_desc_t": "PfSorptionDesc", "pf_prefactor_desc_t": "PfPrefactorDesc",
         "pf_options_t": "PfOptions", "pf_network_desc_t": "PfNetworkDesc", "pf_cell_state_t": "PfCellState",
         "pf_step_stats_t": "PfStepStats", "pf_adjoint_args_t": "PfAdjointArgs", "pf_girt_args_t": "PfGirtArgs",
         "pf_transport_args_t": "PfTransportArgs", "pf_transport_stats_t": "PfTransportStats",
         "pf_constraint_reaction_t": "PfConstraintReaction", "pf_launch_config_t": "PfLaunchConfig"}
KIND = {"integer(c_int32_t)": (4, 4), "integer(c_int64_t)": (8, 8), "real(c_double)": (8, 8),
        "type(c_ptr)": (8, 8)}


def _fortran_source():
    src = open(MODULE).read()
    lines = []
    for raw in src.splitlines():
        line = raw.split("!")[0].rstrip()
        if lines and lines[-1].endswith("&"):
            lines[-1] = lines[-1][:-1] + " " + line.strip().lstrip("&")
        else:
            lines.append(line)
    return lines


def _parameters(lines):
    params = {}
    for line in lines:
        m = re.match(r"\s*integer\(c_int32_t\),\s*parameter.*::(.*)", line, re.I)
        if m:
            for item in m.group(1).split(","):
                k, v = item.split("=")
                params[k.strip().upper()] = int(v)
    return params


def fortran_types():
    """{type name: [(member, kind, count)]} in declaration order."""
    lines = _fortran_source()
    params = _parameters(lines)
    out, cur = {}, None
    for line in lines:
        m = re.match(r"\s*type\s*,\s*bind\(C\)\s*,\s*public\s*::\s*(\w+)", line, re.I)
        if m:
            cur = m.group(1).lower()
            out[cur] = []
            continue
        if cur and re.match(r"\s*end\s+type", line, re.I):
            cur = None
            continue
        if cur and "::" in line:
            spec, names = line.split("::", 1)
            spec = spec.strip().lower().replace(" ", "")
            for nm in re.findall(r"\w+(?:\([^)]*\))?", names):
                mm = re.match(r"(\w+)(?:\(([^)]*)\))?", nm)
                cnt = 1
                if mm.group(2):
                    d = mm.group(2).strip()
                    cnt = int(d) if d.isdigit() else params[d.upper()]
                out[cur].append((mm.group(1).lower(), spec, cnt))
    return out


def fortran_layout(types, name):
    """[(member, offset, size)] and the struct size under C interop rules."""
    off, align_max, res = 0, 1, []
    for member, spec, cnt in types[name]:
        if spec.startswith("type(pf_"):
            sub = spec[5:-1]
            lay, size, al = fortran_layout(types, sub)
        else:
            size, al = KIND[spec]
            size *= cnt
        off = (off + al - 1) // al * al
        res.append((member, off, size))
        off += size
        align_max = max(align_max, al)
    return res, (off + align_max - 1) // align_max * align_max, align_max


def c_members():
    """{struct: [member names]} parsed from the header."""
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\} \1;", src, re.S):
        names = []
        for decl in m.group(2).split(";"):
            decl = " ".join(decl.replace("*", " ").split())
            if not decl:
                continue
            dm = re.match(r"(?:const )?(?:unsigned )?\w+ (.*)$", decl)
            for d in dm.group(1).split(","):
                names.append(re.match(r"\s*(\w+)", d).group(1))
        out[m.group(1)] = names
    return out


@pytest.fixture(scope="module")
def c_offsets():
    gcc = shutil.which("gcc") or shutil.which("cc")
    if not gcc:
        pytest.skip("no C compiler")
    members = c_members()
    body = ["#include <stdio.h>", "#include <stddef.h>", '#include "pfgpu.h"', "int main(void) {"]
    for f, c in TYPES.items():
        body.append('printf("%s size %%zu\\n", sizeof(%s));' % (c, c))
        for mbr in members[c]:
            body.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (c, mbr, c, mbr))
    body.append("return 0; }")
    d = tempfile.mkdtemp()
    try:
        src = os.path.join(d, "off.c")
        open(src, "w").write("\n".join(body))
        exe = os.path.join(d, "off")
        subprocess.run([gcc, "-I", os.path.dirname(HEADER), src, "-o", exe], check=True)
        txt = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    finally:
        shutil.rmtree(d)
    res = {}
    for line in txt.splitlines():
        s, m, v = line.split()
        res.setdefault(s, {})[m] = int(v)
    return members, res


def test_every_header_struct_has_a_fortran_type():
    c = set(c_members())
    assert c == set(TYPES.values()), c ^ set(TYPES.values())
    assert set(fortran_types()) == set(TYPES)


@pytest.mark.parametrize("ftype", sorted(TYPES))
def test_fortran_type_matches_c_struct(c_offsets, ftype):
    members, offs = c_offsets
    cname = TYPES[ftype]
    types = fortran_types()
    lay, size, _ = fortran_layout(types, ftype)
    assert [m for m, _, _ in lay] == [m.lower() for m in members[cname]], (ftype, cname)
    for (m, off, _), cm in zip(lay, members[cname]):
        assert off == offs[cname][cm], (ftype, m, off, offs[cname][cm])
    assert size == offs[cname]["size"], (ftype, size, offs[cname]["size"])


def test_interfaces_match_prototypes():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    protos = {}
    for m in re.finditer(r"\n(?:int32_t|const char\*)\s+(pf_\w+)\((.*?)\);", src, re.S):
        args = [a for a in m.group(2).replace("\n", " ").split(",") if a.strip() and a.strip() != "void"]
        protos[m.group(1)] = len(args)
    text = " ".join(_fortran_source())
    fort = {}
    for m in re.finditer(r"function\s+(pf_\w+)\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", text, re.I):
        assert m.group(1) == m.group(3)
        fort[m.group(1)] = len([a for a in m.group(2).split(",") if a.strip()])
    assert set(fort) == set(protos), set(fort) ^ set(protos)
    for k, v in protos.items():
        assert fort[k] == v, (k, fort[k], v)

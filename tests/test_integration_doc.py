"""The Julia binding written out in INTEGRATION.md must match the C ABI: each
Julia struct's fields, in order and by type, equal the ctypes layout the
library's tests already pin against include/gbde.h; the enum values it uses
equal gbde.h's."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

JULIA_TO_CTYPES = {"Int32": C.c_int32, "Int64": C.c_int64, "UInt64": C.c_uint64,
                   "Float64": C.c_double, "Float32": C.c_float, "Cstring": C.c_char_p}


def julia_code():
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return "\n".join(re.findall(r"```julia\n(.*?)```", doc, flags=re.S))


def julia_structs():
    out = {}
    for name, body in re.findall(r"(?:mutable\s+)?struct\s+(\w+)\s*\n(.*?)\nend", julia_code(),
                                 flags=re.S):
        fields = []
        for line in body.splitlines():
            line = line.split("#")[0]
            if "=" in line and "::" not in line.split("=")[0]:
                continue  # inner constructor
            fields += re.findall(r"(\w+)::([\w{}]+)", line)
        out[name] = fields
    return out


def _same_type(jl, ct):
    if jl.startswith("Ptr{"):
        return ct in (C.c_void_p,) or (isinstance(ct, type) and issubclass(ct, C._Pointer))
    return JULIA_TO_CTYPES[jl] is ct


@pytest.mark.parametrize("jname,cname", [("GbdeProblem", "Problem"), ("GbdeOpts", "Opts"),
                                         ("GbdeOutputs", "Outputs"), ("GbdeCallback", "Callback"),
                                         ("GbdeUserModel", "UserModel")])
def test_julia_struct_matches_abi(capi, jname, cname):
    js = julia_structs()
    assert jname in js, sorted(js)
    jf = js[jname]
    cf = getattr(capi, cname)._fields_
    assert [n for n, _ in jf] == [n for n, _ in cf], jname
    for (n, jt), (_, ct) in zip(jf, cf):
        assert _same_type(jt, ct), (jname, n, jt, ct)


def test_julia_enums_match_header(capi):
    code = julia_code()
    assert "const GBDE_ABI = %d" % capi.lib().gbde_version() in code
    algs = dict((k, int(v)) for k, v in re.findall(r"algid\(::(\w+)\)\s*=\s*(\d+)", code))
    expect = {"Tsit5": capi.ALG_TSIT5, "Vern7": capi.ALG_VERN7,
              "Rosenbrock23": capi.ALG_ROSENBROCK23, "Rodas5": capi.ALG_RODAS5,
              "Rodas5P": capi.ALG_RODAS5P, "EM": capi.ALG_EM, "SOSRI": capi.ALG_SOSRI,
              "SRIW1": capi.ALG_SRIW1}
    assert algs == expect
    # AutoTsit5(stiff): the switching composites; the stiff_threshold option: AUTO
    comp = re.search(r"algid\(alg::OrdinaryDiffEq\.CompositeAlgorithm\) =(.*?)error", code, re.S)
    assert comp and re.findall(r"isa (\w+) \? (\d+)", comp.group(1)) == [
        ("Rosenbrock23", str(capi.ALG_AUTOTSIT5_ROSENBROCK23)),
        ("Rodas5", str(capi.ALG_AUTOTSIT5_RODAS5))]
    assert re.search(r"solver_id\(alg, ea\) = .*: (\d+)", code).group(1) == str(capi.ALG_AUTO)
    prec = dict(re.findall(r":(\w+) => (\d+)", re.search(r"PRECISION = Dict\((.*?)\)", code).group(1)))
    assert {k: int(v) for k, v in prec.items()} == {"fp64": capi.PREC_FP64,
                                                    "mixed": capi.PREC_MIXED,
                                                    "f32x2": capi.PREC_F32X2}
    learned = dict(re.findall(r":(\w+) => (\d+)", re.search(r"LEARNED = Dict\((.*?)\)", code).group(1)))
    assert {k: int(v) for k, v in learned.items()} == {"start": capi.LEARN_START,
                                                       "order": capi.LEARN_ORDER,
                                                       "stiff": capi.LEARN_STIFF}
    rets = dict((int(c), n) for c, n in re.findall(r"c == (\d+) && return ReturnCode\.(\w+)", code))
    assert rets == {capi.RET_SUCCESS: "Success", capi.RET_MAXITERS: "MaxIters",
                    capi.RET_DTLESSTHANMIN: "DtLessThanMin", capi.RET_UNSTABLE: "Unstable",
                    capi.RET_INITIALFAILURE: "InitialFailure", capi.RET_TERMINATED: "Terminated",
                    capi.RET_DEFAULT: "Default"}

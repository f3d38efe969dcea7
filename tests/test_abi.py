"""The C ABI library loads and exports every entry point the headers declare
(no compute calls: this runs without a GPU)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(fg_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_headers_declare_entry_points():
    names = declared_functions()
    for n in ("fg_plan_create", "fg_assemble_fp64", "fg_assemble_mixed", "fg_batch_run", "fg_problem_create"):
        assert n in names


def test_library_exports_all_declared(femg):
    L = femg.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
    assert set(declared_functions()) == set(femg.exported_symbols())


def test_plan_without_device_fails_loudly(femg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    prob = femg.Problem(femg.config_c2(m=1))
    with pytest.raises(femg.FgError) as e:
        prob.plan()
    assert e.value.status == femg.FG_ERR_NO_DEVICE


def test_problem_errors(femg):
    cfg = femg.config_c2(m=1)
    cfg.dim = 4
    with pytest.raises(femg.FgError) as e:
        femg.Problem(cfg)
    assert e.value.status == femg.FG_ERR_ARG

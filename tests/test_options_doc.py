"""Every context option phj_ctx_set_int accepts (csrc/api.cu) is described
in the C ABI header (include/phj_gpu.h), and every option the header
describes is accepted: the two lists stay in step."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def set_int_options():
    src = open(os.path.join(ROOT, "phj-bench_gb300", "csrc", "api.cu")).read()
    body = src[src.index("phj_status phj_ctx_set_int("):]
    body = body[:body.index("\n}\n")]
    return set(re.findall(r'std::strcmp\(name, "([a-z0-9_]+)"\) == 0', body))


def header_options():
    h = open(os.path.join(ROOT, "include", "phj_gpu.h")).read()
    block = h[h.index("/* Integer options of a context:"):h.index("phj_status phj_ctx_set_int(")]
    names = set()
    # an entry opens a line with one or more quoted names, then a colon
    for heads in re.findall(r'^ \*   ((?:"[a-z0-9_]+"(?:, )?)+):', block, flags=re.M):
        names.update(re.findall(r'"([a-z0-9_]+)"', heads))
    return names


def test_every_option_is_documented_and_accepted():
    accepted, documented = set_int_options(), header_options()
    assert accepted, "no options parsed from phj_ctx_set_int"
    assert accepted - documented == set(), f"accepted but not described in the header: {sorted(accepted - documented)}"
    assert documented - accepted == set(), f"described in the header but not accepted: {sorted(documented - accepted)}"

"""The oracle recipe's amalgamation step (oracle/build.py: amalgamate): a
translation unit with every include that resolves in the given directories
inlined, so the reference builds and the FleCSI wrapper build compile on a host
without the reference checkout.  Checked on a small tree of headers: quoted
includes resolve beside the including file first, then in the directories in
order; angle includes only in the directories; headers found nowhere stay
include lines; a #pragma once header is inlined once; #line directives keep the
sources' names and lines; and the result compiles to the same program."""
import os
import runpy
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ob():
    return runpy.run_path(os.path.join(ROOT, "oracle", "build.py"), run_name="oracle_build")


def _tree(tmp):
    files = {
        "src/main.cc": '#include <cstdio>\n#include "local.hh"\n#include <lib/api.hh>\n#include "lib/api.hh"\n'
                       'int main() { std::printf("%d\\n", local() + api()); return 0; }\n',
        "src/local.hh": "#pragma once\ninline int local() { return 40; }\n",
        "shim/lib/api.hh": '#pragma once\n#include "detail.hh"\ninline int api() { return detail(); }\n',
        "shim/lib/detail.hh": "#ifndef DETAIL_HH\n#define DETAIL_HH\ninline int detail() { return 2; }\n#endif\n",
        "ref/lib/api.hh": "#error the shim's api.hh comes first\n",
    }
    for rel, text in files.items():
        path = os.path.join(tmp, rel)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            f.write(text)
    return os.path.join(tmp, "src", "main.cc"), [os.path.join(tmp, "shim"), os.path.join(tmp, "ref")]


def test_amalgamate_inlines_what_resolves_and_keeps_the_rest(ob, tmp_path):
    src, dirs = _tree(str(tmp_path))
    text = ob["amalgamate"](src, dirs, os.path.basename)
    lines = text.splitlines()
    assert [x for x in lines if x.startswith("#include")] == ["#include <cstdio>"]
    assert text.count("inline int api()") == 1  # #pragma once: the second include adds nothing
    assert text.count("inline int detail()") == 1
    assert "#error" not in text  # the shim directory comes before the reference's
    assert "#pragma once" not in text
    assert '#line 1 "local.hh"' in lines and '#line 1 "api.hh"' in lines
    # after an inlined header the including file's numbering resumes at the next line
    i = lines.index('#line 1 "local.hh"')
    assert lines[i + 3] == '#line 3 "main.cc"'


def test_amalgamated_unit_compiles_to_the_same_program(ob, tmp_path):
    src, dirs = _tree(str(tmp_path))
    unit = os.path.join(str(tmp_path), "unit.cc")
    with open(unit, "w") as f:
        f.write(ob["amalgamate"](src, dirs, os.path.basename))
    exe = os.path.join(str(tmp_path), "a.out")
    subprocess.run(["g++", "-std=c++17", unit, "-o", exe], check=True)  # no -I: everything is inlined
    assert subprocess.run([exe], capture_output=True, text=True, check=True).stdout.strip() == "42"

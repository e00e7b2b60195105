"""The commands the documentation and the profile summaries quote still run.

Every `python bench.py …` in the Markdown files parses with bench.py's own
argument parser, every `python -m <module>` names an importable module, and
every `python <file>.py` names a file of the repository.  CPU only: nothing is
executed.
"""

import importlib.util
import re
import shlex
from pathlib import Path

import pytest

from conftest import REPO

DOCS = sorted(Path(REPO, "profiles").glob("*.md")) + [
    Path(REPO, n) for n in ("DESIGN.md", "INTEGRATION.md", "README.md")
]
CMD = re.compile(r"python3? ([^`\n|&>;#\\]+)")


def quoted_commands():
    out = []
    for doc in DOCS:
        for m in CMD.finditer(doc.read_text()):
            text = m.group(1).strip()
            if text.startswith("-c"):  # inline programs are cut at their first ';'
                continue
            out.append((doc.name, shlex.split(text, posix=True)))
    return out


COMMANDS = quoted_commands()


def test_the_docs_quote_benchmark_commands():
    assert sum(1 for _, a in COMMANDS if a[0] == "bench.py") >= 8


@pytest.mark.parametrize("doc,argv", COMMANDS, ids=[f"{d}:{' '.join(a)}" for d, a in COMMANDS])
def test_quoted_command_is_valid(doc, argv):
    if argv[0] == "bench.py":
        import bench

        bench.arg_parser().parse_args(argv[1:])
    elif argv[0] == "-m":
        mod = argv[1]
        if mod == "pytest":
            return
        assert importlib.util.find_spec(mod) is not None, f"{doc}: no module {mod}"
    else:
        assert Path(REPO, argv[0]).is_file(), f"{doc}: no file {argv[0]}"

"""The committed measurement summaries: each names its command (ncu or a
plain timing run), the command runs committed files only, and every ncu
invocation leaves the clocks alone."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _commands(path):
    txt = open(path).read()
    return txt, re.findall(r"```\n(.*?)```", txt, re.S)


def test_every_summary_has_a_command_on_committed_files():
    paths = sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md")))
    assert paths
    for p in paths:
        txt, blocks = _commands(p)
        cmd = "\n".join(b for b in blocks if "ncu" in b or "python" in b)
        assert cmd, os.path.basename(p)
        assert "_work/" not in cmd, os.path.basename(p)
        runs = [m for m in re.finditer(r"(?m)^\s*ncu\s+(?!-i\b)", cmd)]
        assert len(runs) == cmd.count("--clock-control none"), os.path.basename(p)
        for mod in re.findall(r"python\s+-m\s+(\S+)", cmd):
            if mod.startswith("thecodecombo_7_gb300"):  # the project's own modules
                assert os.path.exists(os.path.join(ROOT, *mod.split(".")) + ".py"), mod
        for script in re.findall(r"python\s+(\S+\.py)", cmd):
            assert os.path.exists(os.path.join(ROOT, script)), (os.path.basename(p), script)

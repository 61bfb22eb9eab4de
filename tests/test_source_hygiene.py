"""Source rules for the CUDA library, checked on the text of the sources (CPU only):

* no kernel stops itself with a trap or a device-side assert: failures are reported through the
  int status and the status words the kernels write, so a bad input never takes the context down;
* no source calls or names the batched memory-copy entry points of the CUDA runtime and driver
  (one plain asynchronous copy per buffer is used instead); the names are assembled here so that
  this file does not contain them either;
* every spin-wait on an mbarrier has an iteration limit.
"""
import glob
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(REPO, "pibronic_gb300", "csrc")


def _sources(exts=(".cu", ".cuh", ".h", ".py")):
    roots = [os.path.join(REPO, d) for d in ("pibronic_gb300", "include", "oracle", "tests")]
    roots.append(REPO)
    out = set()
    for root in roots:
        pattern = "**/*" if root != REPO else "*"
        for path in glob.glob(os.path.join(root, pattern), recursive=root != REPO):
            if path.endswith(exts) and "_work" not in path:
                out.add(path)
    return sorted(out)


def test_no_trap_or_device_assert_in_kernels():
    for path in glob.glob(os.path.join(CSRC, "*.cu*")):
        text = open(path).read()
        assert "__trap" not in text, path
        assert not re.search(r"(?<![A-Za-z_])assert\s*\(", text), path
        assert "trap;" not in text, path


def test_no_batched_copy_entry_points():
    names = [p + "Memcpy" + d + "BatchAsync" for p in ("cuda", "cu") for d in ("", "3D")]
    for path in _sources():
        text = open(path, errors="replace").read()
        for name in names:
            assert name not in text, (path, name)


def test_mbarrier_waits_are_bounded():
    for path in glob.glob(os.path.join(CSRC, "*.cu*")):
        text = open(path).read()
        for m in re.finditer(r"mbarrier\.try_wait", text):
            window = text[max(0, m.start() - 600):m.start()]
            assert re.search(r"for\s*\(\s*uint32_t\s+\w+\s*=\s*0;\s*\w+\s*<\s*kSpinLimit", window), \
                (path, text.count("\n", 0, m.start()) + 1)

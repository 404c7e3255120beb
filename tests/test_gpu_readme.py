"""The README's Python example runs as written and its results agree with
the oracle."""
import os
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_readme_example(oracle, gpu):
    text = open(os.path.join(ROOT, "README.md")).read()
    blocks = re.findall(r"```python\n(.*?)```", text, re.S)
    assert blocks, "README has a Python example"
    ns = {}
    exec(compile(blocks[0], "README.md", "exec"), ns)
    x, image = ns["x"], ns["image"]
    assert image == oracle.encode(x, 10000)
    words, cnt = oracle.range_filter(image, 10000, 1.05)[:2]
    assert ns["hits"].count == cnt and np.array_equal(ns["hits"].words, words)
    assert ns["total"] == oracle.buff_sum(image, 10000)[0]
    assert np.array_equal(ns["values"], oracle.decode(image, 10000))
    bitmap, s = ns["bitmap"], ns["s"]
    assert bitmap.count == cnt and s.sum == ns["total"]

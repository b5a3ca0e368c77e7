"""Host side of the serving loop without a GPU: the admission estimate and the
C/ctypes layout of the request, result and statistics records."""
import os
import subprocess

import pytest

from tests import decks

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def A():
    from epic2d_mcc_gb300 import build as B

    B.build()
    from epic2d_mcc_gb300 import api

    return api


def test_record_layouts_match_the_header(A, tmp_path):
    import ctypes

    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include "epic2d_serve.h"\nint main(void){printf("%zu %zu %zu\\n",'
                   ' sizeof(epic_request), sizeof(epic_result), sizeof(epic_server_stats)); return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [ctypes.sizeof(A.Request), ctypes.sizeof(A.Result), ctypes.sizeof(A.ServerStats)]


def test_estimate_grows_with_the_run(A, tmp_path):
    d = str(tmp_path)
    small = A.make_request(decks.write(decks.deck(nx=64, ny=64, ne=40000, ni=40000), d), 10)
    big = A.make_request(decks.write(decks.deck(nx=64, ny=64, ne=400000, ni=400000), d), 10)
    grid = A.make_request(decks.write(decks.deck(nx=256, ny=256, ne=40000, ni=40000), d), 10)
    e_small, e_big, e_grid = A.estimate_bytes(small), A.estimate_bytes(big), A.estimate_bytes(grid)
    assert 0 < e_small < e_big and e_small < e_grid
    # at least the particle arrays: 2 species x capacity x 40 B (FP64 form)
    assert e_big >= 2 * (400000 * 3 // 2) * 40
    mixed = A.make_request(decks.write(decks.deck(nx=64, ny=64, ne=400000, ni=400000), d), 10, precision=1)
    assert A.estimate_bytes(mixed) < e_big
    coll = A.make_request(decks.write(decks.deck(nx=64, ny=64, ne=400000, ni=400000), d), 10, collisions=True)
    assert A.estimate_bytes(coll) > e_big
    sorted_ = A.make_request(decks.write(decks.deck(nx=64, ny=64, ne=400000, ni=400000), d), 10, sort_every=16)
    assert A.estimate_bytes(sorted_) > e_big

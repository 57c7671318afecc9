"""The noise oracle's Philox4x32-10 against the algorithm's published known
answer (counter 0, key 0; Random123 test vectors), and its normals' moments."""

import numpy as np

from oracle import nlse_oracle as orc


def test_philox_known_answer():
    z = np.zeros(1, np.uint64)
    out = [int(x[0]) for x in orc.philox4x32_10((z, z, z, z), 0, 0)]
    assert out == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]


def test_noise_moments():
    n0, n1 = orc.ddgpe_noise(1 << 16, 3, 17)
    for n in (n0, n1):
        for part in (n.real, n.imag):
            assert abs(part.mean()) < 0.02 and abs(part.std() - 1) < 0.02

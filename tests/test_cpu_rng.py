"""The numpy restatement of the thermostats' Philox4x32-10 generator against the
known-answer vectors published with the paper's Random123 library (Salmon et al., SC'11):
counter and key all zeros, all ones, and the hexadecimal digits of pi."""
import numpy as np

from oracle.philox import philox4x32_10, uniforms

KAT = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF), (0xFFFFFFFF, 0xFFFFFFFF),
     (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def test_philox_known_answers():
    for ctr, key, want in KAT:
        got = philox4x32_10(np.array([ctr], np.uint32), key)[0]
        assert tuple(int(x) for x in got) == want, [hex(int(x)) for x in got]


def test_uniforms_cover_half_open_interval():
    u = uniforms(7, 3, 11, 1, 1 << 16)
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 5 * np.sqrt(1 / 12 / u.size)

"""The device rand() stream's algorithm (the C library's rand() after
srand(seed), restated in tm_libcrand.cu) against the C library itself, on the
host: no GPU needed."""
import numpy as np


def test_libc_rand_stream_restatement():
    """The device rand() stream's algorithm (tmi_libc_rand_host runs it on the
    host, chunk by chunk and with the same jump-ahead as the device): the C
    library's own values after srand(seed), for seeds at the edges of the
    seeding arithmetic and offsets that take the jump-ahead path."""
    import ctypes

    from timothy_gb300.session import LIB_PATH

    lib = ctypes.CDLL(LIB_PATH)
    libc = ctypes.CDLL(None)
    libc.srand.argtypes = [ctypes.c_uint]
    libc.rand.restype = ctypes.c_int
    lib.tmi_libc_rand_host.argtypes = [ctypes.c_uint32, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]
    for seed in (0, 1, 31, 2 ** 31 - 1, 2 ** 31, 2 ** 32 - 1):
        for off, cnt in ((0, 5000), (40000, 4500)):
            libc.srand(seed)
            for _ in range(off):
                libc.rand()
            ref = np.array([libc.rand() for _ in range(cnt)], np.int32)
            out = np.zeros(cnt, np.int32)
            lib.tmi_libc_rand_host(seed, off, cnt, out.ctypes.data)
            assert np.array_equal(out, ref), (seed, off)

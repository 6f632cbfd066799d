"""Generate tests/golden/philox_curand.json: raw Philox4x32-10 output of
cuRAND's host generator (CURAND_RNG_PSEUDO_PHILOX4_32_10, run on the CPU),
an implementation independent of this repository.  cuRAND's sequential
output block k of seed s is Philox(key = s, counter = (0, 0, k, 0)).

Run where libcurand is available: python tests/golden/make_philox_vectors.py
"""
import ctypes as C
import json
import os

CURAND = os.environ.get("CURAND_LIB", "/usr/local/cuda/lib64/libcurand.so")


def main():
    L = C.CDLL(CURAND)
    out = []
    for seed in (0x0123456789ABCDEF, 1, 0xDEADBEEF, 2 ** 63 + 12345):
        g = C.c_void_p()
        assert L.curandCreateGeneratorHost(C.byref(g), 161) == 0  # PHILOX4_32_10
        assert L.curandSetPseudoRandomGeneratorSeed(g, C.c_ulonglong(seed)) == 0
        buf = (C.c_uint32 * 64)()
        assert L.curandGenerate(g, buf, C.c_size_t(64)) == 0
        L.curandDestroyGenerator(g)
        words = list(buf)
        out.append({"seed": seed, "blocks": [{"counter": [0, 0, k, 0],
                                              "out": words[4 * k:4 * k + 4]}
                                             for k in range(16)]})
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "philox_curand.json")
    with open(path, "w") as f:
        json.dump({"source": "cuRAND host generator CURAND_RNG_PSEUDO_PHILOX4_32_10",
                   "vectors": out}, f, indent=1)
    print(path)


if __name__ == "__main__":
    main()

"""Generate chacha20_openssl.json: ChaCha20 keystream blocks from OpenSSL (via `cryptography`).

These pin the ChaCha block function that StdRng (ChaCha12, rand_chacha 0.3.1) is built on: the
tests run the oracle's and the library's block function at 20 rounds on the same key, 64-bit block
counter and 64-bit stream, and compare with OpenSSL.  OpenSSL's 16-byte ChaCha20 "nonce" is the
little-endian state words 12..15, i.e. counter (low, high) then stream (low, high) in the layout
rand_chacha uses.  Keys include rand_core's PCG32 seed_from_u64 expansion of a few seeds, so the
vectors exercise the exact keys make_offsets (src/rng.rs:15) feeds the block function.

Run:  python tests/golden/make_chacha_vectors.py   (needs the `cryptography` package)
"""
import json
import os
import struct

from cryptography.hazmat.primitives.ciphers import Cipher, algorithms

M64 = (1 << 64) - 1


def pcg32_key(state: int):
    key = []
    for _ in range(8):
        state = (state * 6364136223846793005 + 11634580027462260723) & M64
        xs = (((state >> 18) ^ state) >> 27) & 0xFFFFFFFF
        rot = state >> 59
        key.append(((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF)
    return key


def block(key_words, counter, stream):
    key = struct.pack("<8I", *key_words)
    nonce = struct.pack("<QQ", counter, stream)
    enc = Cipher(algorithms.ChaCha20(key, nonce), mode=None).encryptor()
    ks = enc.update(b"\x00" * 64)
    return list(struct.unpack("<16I", ks))


def main():
    cases = []
    keys = [pcg32_key(s) for s in (0, 1, 42, 5489, 0x9E3779B97F4A7C15, M64)]
    keys.append([0] * 8)
    keys.append(list(range(8)))
    for ki, key in enumerate(keys):
        for counter, stream in ((0, 0), (1, 0), (7, 0), (0xFFFFFFFE, 0), (3, 0x0123456789ABCDEF)):
            cases.append({"key": key, "counter": counter, "stream": stream, "block": block(key, counter, stream)})
    seeds = [0, 1, 42, 5489, 0x9E3779B97F4A7C15, M64]
    out = {"source": "OpenSSL ChaCha20 via cryptography", "rounds": 20, "cases": cases,
           "pcg32_keys": [{"seed": s, "key": pcg32_key(s)} for s in seeds]}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "chacha20_openssl.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1)
    print(path, len(cases))


if __name__ == "__main__":
    main()

"""Stand-in so lettuce imports in a container without this optional
dependency; it is not on lettuce's arithmetic path (file output / module
naming only). ``hash_bytes`` names lettuce's generated cuda_native modules
(lettuce/cuda_native/_util.py:6-9): any digest that differs between
configurations serves, so this one is BLAKE2b, not MurmurHash3."""
import hashlib


def hash(*a, **k):
    return 0


def hash_bytes(value, *a, **k):
    if isinstance(value, str):
        value = value.encode()
    return hashlib.blake2b(bytes(value), digest_size=16).digest()

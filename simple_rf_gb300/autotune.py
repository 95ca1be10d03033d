"""The library's online tile-shape tuner (srf_autotune_*): switch it on or off, list
the choices it has made, and save / preload them as JSON so that a later process
starts from the same shapes without timing them again."""
import ctypes
import json

from . import _lib

SITES = {1: 'gemm_epilogue_warps', 2: 'basis_encode_tile', 3: 'vm_color_group'}


def enable(on=True):
    _lib.check(_lib.load().srf_autotune_enable(int(bool(on))), 'srf_autotune_enable')


def clear():
    _lib.check(_lib.load().srf_autotune_clear(), 'srf_autotune_clear')


def table():
    """[{'site', 'key': (a, b, c), 'choice'}] for every tuned shape."""
    lib = _lib.load()
    out = []
    for i in range(lib.srf_autotune_count()):
        site, choice = ctypes.c_int(), ctypes.c_int()
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(lib.srf_autotune_entry(i, ctypes.byref(site), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                          ctypes.byref(choice)), 'srf_autotune_entry')
        out.append({'site': site.value, 'site_name': SITES.get(site.value, '?'), 'key': (a.value, b.value, c.value),
                    'choice': choice.value})
    return out


def save(path):
    with open(path, 'w') as f:
        json.dump(table(), f, indent=1)


def load(path):
    lib = _lib.load()
    with open(path) as f:
        for e in json.load(f):
            a, b, c = e['key']
            _lib.check(lib.srf_autotune_set(int(e['site']), int(a), int(b), int(c), int(e['choice'])),
                       'srf_autotune_set')

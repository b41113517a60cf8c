"""The reference's own CPU core (oracle/_ref/libkodama_ref.so, compiled from the
reference sources by oracle/build_ref.sh).  TEST INFRASTRUCTURE ONLY: present
only where the reference checkout exists; pins the CPU restatement and makes
the tests/golden fixtures."""

from __future__ import annotations

import functools
import os

from . import bindings as _b

_LIB = _b._Lib(os.path.join(_b._HERE, "_ref", "libkodama_ref.so"), "ref_")


def available() -> bool:
    return _LIB.available()


def _bind(fn):
    return functools.partial(fn, _LIB)


kodama_matrix_graph_data = _bind(_b.kodama_matrix_graph_data)
kodama_matrix_raw = _bind(_b.kodama_matrix_raw)
core_knn_graph = _bind(_b.core_knn_graph)
dissimilarity = _bind(_b.dissimilarity)
plsldacv = _bind(_b.plsldacv)
plsldapredict = _bind(_b.plsldapredict)
knncv = _bind(_b.knncv)
core_plslda = _bind(_b.core_plslda)
core_knn = _bind(_b.core_knn)

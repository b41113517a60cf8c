"""CPU restatement of the KODAMA.matrix hot path (oracle/kodama_oracle.cpp,
built into oracle/_build/liboracle.so by oracle/build_oracle.sh).

TEST INFRASTRUCTURE ONLY: the checker the CUDA path is compared against in
tests/, in __graft_entry__.smoke() and as bench.py's CPU baseline.  The product
(kodama_gb300) never imports it."""

from __future__ import annotations

import functools
import os
import subprocess

from . import bindings as _b

_LIB = _b._Lib(os.path.join(_b._HERE, "_build", "liboracle.so"), "orc_")


def build() -> None:
    subprocess.run([os.path.join(_b._HERE, "build_oracle.sh")], check=True)


def available() -> bool:
    return _LIB.available()


def _bind(fn):
    return functools.partial(fn, _LIB)


kodama_matrix_graph_data = _bind(_b.kodama_matrix_graph_data)
core_knn_graph = _bind(_b.core_knn_graph)
dissimilarity = _bind(_b.dissimilarity)
exact_knn = _bind(_b.exact_knn)
exact_knn_rows = _bind(_b.exact_knn_rows)
exact_knn_metric = _bind(_b.exact_knn_metric)
kmeans = _bind(_b.kmeans)
dot_x86 = _bind(_b.dot_x86)
quota_sample = _bind(_b.quota_sample)
core_plslda = _bind(_b.core_plslda)
plsldacv = _bind(_b.plsldacv)
plsldapredict = _bind(_b.plsldapredict)
knncv = _bind(_b.knncv)
core_knn = _bind(_b.core_knn)

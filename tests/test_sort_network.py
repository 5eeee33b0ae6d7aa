"""The 25-comparator network that orders each lane's nine stencil rows longest
first (sort_row_keys in flowx_gb300/csrc/neighbour.cuh). Any comparator
network permutes its inputs, so the neighbour walks test every row once
whatever the network; this checks that it also sorts, read from the CUDA
source and run on all 2^9 inputs of zeros and ones (a network that sorts
those sorts every input)."""

import itertools
import os
import re

SRC = os.path.join(os.path.dirname(__file__), "..", "flowx_gb300", "csrc", "neighbour.cuh")


def _network():
    text = open(SRC).read()
    start = text.index("void sort_row_keys(")
    body = text[start:text.index("\n}\n", start)]
    return [(int(a), int(b)) for a, b in re.findall(r"row_key_exchange\(key\[(\d)\], key\[(\d)\]\)", body)]


def test_row_key_network_sorts_descending():
    net = _network()
    assert len(net) == 25
    for bits in itertools.product((0, 1), repeat=9):
        v = list(bits)
        for a, b in net:
            # row_key_exchange: the larger key first
            if v[a] < v[b]:
                v[a], v[b] = v[b], v[a]
        assert v == sorted(bits, reverse=True), bits

"""Serialised indexes: a tree written by knn_index_serialize and read back by
knn_index_deserialize answers every query exactly as the original (and as the oracle), with its
learned-radius model; a damaged blob is rejected."""

import numpy as np
import pytest

import oracle
from cudaexactknn_gb300 import _lib, knn, workloads as W

pytestmark = pytest.mark.gpu

gu = pytest.importorskip("gpu_util")


@pytest.mark.parametrize("structure,dims,skips", [("bf", 3, 0), ("bf", 128, 0), ("kd", 3, 0), ("kd", 8, 2),
                                                  ("ball", 16, 1), ("ball", 32, 3)])
def test_round_trip_matches_the_original(structure, dims, skips):
    rng = np.random.default_rng(dims + skips)
    pts = W.uniform(rng, 30000, dims)
    qs = W.uniform(rng, 2000, dims)
    k = 10
    want = oracle.bf_knn(pts, qs, k, fma=True, threads=8)
    ix = gu.make_index(structure, pts, skips)
    blob = ix.serialize()
    info = ix.info()
    ix.close()
    back = knn.load_index(blob)
    got_info = back.info()
    for f in ("structure", "n", "dims", "aux_dims", "depth_skips", "node_depth", "leaf_slots", "node_count"):
        assert getattr(got_info, f) == getattr(info, f), f
    gu.assert_rows_equal(*gu.run(back, qs, k), *want, what=f"{structure} loaded")
    # Serialising the loaded index gives the same bytes.
    assert back.serialize() == blob
    back.close()


def test_round_trip_keeps_the_radius_model():
    rng = np.random.default_rng(5)
    pts, centres = W.mixture(rng, 50000, 3, 16, 0.02)
    qs, _ = W.mixture(rng, 4000, 3, 16, 0.02, centres)
    train, _ = W.mixture(rng, 8192, 3, 16, 0.02, centres)
    k = 16
    ix = gu.make_index("kd", pts, 0)
    ix.train_radius_model(gu.to_dev(train), k, steps=300)
    blob = ix.serialize()
    seeded = gu.run(ix, qs, k, flags=_lib.QF_LEARNED_RADIUS)
    ix.close()
    back = knn.load_index(blob)
    assert back.info().radius_model == 1
    got = gu.run(back, qs, k, flags=_lib.QF_LEARNED_RADIUS)
    gu.assert_rows_equal(*got, *seeded, what="learned radius after loading")
    gu.assert_rows_equal(*got, *oracle.bf_knn(pts, qs, k, fma=True, threads=8), what="vs oracle")
    back.close()


def test_damaged_blob_is_rejected():
    rng = np.random.default_rng(9)
    ix = gu.make_index("ball", W.uniform(rng, 5000, 16), 1)
    blob = bytearray(ix.serialize())
    ix.close()
    blob[len(blob) // 2] ^= 0x40
    with pytest.raises(Exception, match="checksum"):
        knn.load_index(bytes(blob))

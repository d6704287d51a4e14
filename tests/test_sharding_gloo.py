"""Column-sharded interaction matrix over 2 gloo ranks on the CPU.

The local measurement is replaced by the float64 oracle's interaction
matrix of a tiny sensor, so the test checks the partition, the gather and
the timing reduction without a GPU: the sharded D must equal the oracle's
single-process D exactly."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _tiny():
    from oracle import pwfs_oracle as O
    res = 24
    pup = O.telescope_pupil(res)
    inten = O.source_intensity(pup, O.n_photon('V0', 8), 1e-3, 8.0)
    w = O.build_pyramid(res, 4, 3, 0.5, inten)
    modes = O.dm_modes(res, 8.0, 4)
    return O, w, modes, pup


def _rank_main(rank, world, port, n_cols, out_dir):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        from oopao_gb300.sharding import column_shards, max_over_ranks, sharded_interaction_matrix
        O, w, modes, pup = _tiny()
        m2c = np.eye(modes.shape[1])[:, :n_cols]
        seen = []

        def column_fn(m):
            seen.append(m.shape[1])
            if m.shape[1] == 0:
                return np.zeros((w.valid_signal.sum(), 0))
            return O.interaction_matrix(w, modes, m, 1e-8, 500e-9, pup, single_pass=False)

        D = sharded_interaction_matrix(None, None, None, None, m2c, 1e-8, single_pass=False, column_fn=column_fn)
        t = max_over_ranks(float(rank + 1))
        s, e = column_shards(n_cols, world)[rank]
        np.savez(os.path.join(out_dir, 'rank%d.npz' % rank), D=D, t=t, width=seen[0], s=s, e=e)
    finally:
        dist.destroy_process_group()


def test_column_shards_balanced():
    from oopao_gb300.sharding import column_shards
    assert column_shards(10, 3) == [(0, 4), (4, 7), (7, 10)]
    assert column_shards(2, 4) == [(0, 1), (1, 2), (2, 2), (2, 2)]
    for n, w in ((300, 8), (1000, 3), (7, 7), (0, 2)):
        sh = column_shards(n, w)
        assert sh[0][0] == 0 and sh[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(sh, sh[1:]))
        widths = [e - s for s, e in sh]
        assert max(widths) - min(widths) <= 1


@pytest.mark.parametrize('n_cols', [7, 1])
def test_sharded_im_equals_single_process(tmp_path, n_cols):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), n_cols, str(tmp_path)), nprocs=world,
                       start_method='spawn')
    O, w, modes, pup = _tiny()
    Dref = O.interaction_matrix(w, modes, np.eye(modes.shape[1])[:, :n_cols], 1e-8, 500e-9, pup,
                                single_pass=False)
    for r in range(world):
        z = np.load(tmp_path / ('rank%d.npz' % r))
        np.testing.assert_array_equal(z['D'], Dref)
        assert float(z['t']) == 2.0                     # max over ranks of rank+1
        assert int(z['width']) == int(z['e']) - int(z['s'])

"""The on-disk dictionary reader against the layout load_dictionary produces (CPU only)."""
import numpy as np

from commit_gb300 import dictionary, synth


def test_round_trip_through_dict_files(tmp_path):
    D, K = synth.make_dictionary(synth.ProblemSpec(dim=(12, 10, 8), n_mask=700, n_fibers=120, ndirs=60,
                                                   shells=[(1000.0, 10)], seed=4))
    mask = D['MASK']
    lin = mask.ravel(order='F').nonzero()[0]           # mask index -> linear grid index
    IC = D['IC']
    rng = np.random.default_rng(0)
    p = rng.permutation(IC['n'])                       # trk2dictionary writes per-thread chunks
    raw = {'IC': {'str': IC['str'][p], 'vox': lin[IC['vox'][p]], 'dir': IC['dir'][p],
                  'len': (IC['len'][p] * D['TRK']['norm'][IC['str'][p]]).astype(np.float32)},
           'EC': {'vox': lin[D['EC']['vox']][::-1], 'dir': D['EC']['dir'][::-1]},
           'ISO': {'vox': lin[D['ISO']['vox']]},
           'TRK': {'norm': D['TRK']['norm'], 'kept': D['TRK']['kept']}}
    dictionary.write_dictionary(str(tmp_path), raw)
    L = dictionary.load_dictionary(str(tmp_path), mask)
    assert L['IC']['n'] == IC['n'] and L['IC']['nSTR'] == IC['nSTR'] and L['IC']['nVOX'] == IC['nVOX']
    assert np.array_equal(L['IC']['vox'], IC['vox'])
    # within a voxel the stable sort keeps the file order; compare as multisets per voxel
    key = lambda d: np.lexsort((d['len'], d['dir'], d['str'], d['vox']))  # noqa: E731
    a, b = key(L['IC']), key(IC)
    for k in ('vox', 'str', 'dir'):
        assert np.array_equal(L['IC'][k][a], IC[k][b])
    np.testing.assert_allclose(L['IC']['len'][a], IC['len'][b], rtol=2e-7)
    assert np.array_equal(np.sort(L['EC']['vox']), np.sort(D['EC']['vox']))
    assert np.array_equal(L['ISO']['vox'], D['ISO']['vox'])
    assert L['MASK_ix'].size == IC['nVOX']

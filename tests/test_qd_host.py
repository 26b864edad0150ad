"""QD glue host logic (leniax lenia.py / qd.py / utils.py), no GPU."""
import torch

from leniax_gb300 import qd


def test_get_config_scales_genes_into_their_domains():
    # the individual of leniax tests/test_qd.py:16-48
    config = {
        'kernels_params': [{'r': 1, 'b': '1', 'm': 0.17, 's': 0.015, 'h': 1, 'k_id': 0, 'gf_id': 0, 'c_in': 0,
                            'c_out': 0}],
        'genotype': [{'key': 'kernels_params.0.m', 'domain': [0., .5], 'type': 'float'},
                     {'key': 'kernels_params.0.s', 'domain': [0., 2.], 'type': 'float'}]
    }
    ind = qd.LeniaIndividual(config, 1, [0.7, 0.3])
    new = ind.get_config()
    assert new['kernels_params'][0]['m'] == 0.35
    assert new['kernels_params'][0]['s'] == 0.6
    assert config['kernels_params'][0]['m'] == 0.17  # the individual works on its own copy


def test_gene_types_and_nested_paths():
    genotype = [{'key': 'kernels_params.0.gf_params.0', 'domain': [0.1, 0.3], 'type': 'float'},
                {'key': 'world_params.T', 'domain': [5, 10], 'type': 'int'},
                {'key': 'kernels_params.0.kf_slug', 'domain': ['gauss_bump', 'poly_quad'], 'type': 'choice'}]
    up = qd.get_update_config(genotype, [0.5, 0.99, 0.9])
    assert abs(up['kernels_params'][0]['gf_params'][0] - 0.2) < 1e-12
    assert up['world_params']['T'] == 10  # int(5 + 6 * 0.99 - 0.5)
    assert up['kernels_params'][0]['kf_slug'] == 'poly_quad'  # domain[int(2 * 0.9 - 0.5)]
    assert qd.get_update_config(genotype[2:], [0.7])['kernels_params'][0]['kf_slug'] == 'gauss_bump'
    d = {'a': [{'b': 1.5}]}
    assert qd.get_param(d, 'a.0.b') == 1.5
    qd.set_param(d, 'a.2.c', 3)
    assert d['a'][2] == {'c': 3} and d['a'][1] == {}


def test_update_individuals_fitness_and_best_inits():
    # leniax tests/test_qd.py:97-118
    cfg = {'algo': {}, 'kernels_params': []}
    inds = [qd.LeniaIndividual(cfg, 1), qd.LeniaIndividual(cfg, 2)]
    out = qd.update_individuals(inds, {'N': torch.tensor([[1, 2, 3], [1, 3, 4]])})
    assert [i.fitness for i in out] == [3, 4]
    assert out[0].qd_config['algo']['best_init_idxs'] == [2]


def test_update_individuals_behaviours_window():
    cfg = {'algo': {}, 'kernels_params': [], 'phenotype': ['behaviours.mass']}
    T = 300
    mass = torch.arange(T, dtype=torch.float32)[None, :, None].repeat(2, 1, 3)  # [Ns, T, Ni]
    mass[1, :, 1] += 1000.
    N = torch.tensor([[200, 150, 10], [50, 250, 250]])
    inds = [qd.LeniaIndividual(cfg, 1), qd.LeniaIndividual(cfg, 2)]
    qd.update_individuals(inds, {'N': N, 'mass': mass})
    # individual 0: ns = 200, window [72, 200) of init 0 -> mean 135.5
    assert abs(inds[0].features[0] - 135.5) < 1e-9
    # individual 1: ns = 250, first best init 1 -> window [122, 250) + 1000
    assert abs(inds[1].features[0] - (1000. + 185.5)) < 1e-9
    assert inds[1].qd_config['algo']['best_init_idxs'] == [1, 2]


def test_stats_list_to_dict_and_flat_kernel_params():
    # statistics.py:339-360: per-step dicts (floats or arrays) -> per-key arrays over the steps
    import torch
    from leniax_gb300 import kernels, statistics
    steps = [{'mass': 1.0, 'channel_mass': torch.tensor([0.5, 0.5])}, {'mass': 2.0, 'channel_mass': torch.tensor([1., 1.])}]
    d = statistics.stats_list_to_dict(steps)
    assert d['mass'].tolist() == [1.0, 2.0] and tuple(d['channel_mass'].shape) == (2, 2)
    assert statistics.stats_list_to_dict([]) == {}
    # kernels.py:38-45: the kernel params in the mapping's channel-sorted order
    kp = [{'k_slug': 'circle_2d', 'k_params': [1.0, [1.0]], 'kf_slug': 'gauss_bump', 'kf_params': [4.0],
           'gf_slug': 'gaussian', 'gf_params': [0.15, 0.015], 'h': 1.0, 'c_in': 1, 'c_out': 0},
          {'k_slug': 'circle_2d', 'k_params': [0.5, [1.0, 0.5]], 'kf_slug': 'gauss_bump', 'kf_params': [4.0],
           'gf_slug': 'gaussian', 'gf_params': [0.2, 0.02], 'h': 1.0, 'c_in': 0, 'c_out': 1}]
    _, mp = kernels.get_kernels_and_mapping(kp, [32, 32], 2, 8.0, True, torch.device('cpu'))
    assert mp.get_k_params() == [[0.5, [1.0, 0.5]], [1.0, [1.0]]]
    assert mp.get_gf_params().tolist() == [[0.20000000298023224, 0.019999999552965164], [0.15000000596046448,
                                                                                       0.014999999664723873]]

import numpy as np

from tangerine_gb300 import workloads as W


def test_generator_is_seeded_and_stable():
    a = W.random_tree(3, 256)
    b = W.random_tree(3, 256)
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, W.random_tree(4, 256))
    assert W.spec_primitive_count(a) == 256


def test_mt19937_words_match_the_standard_sequence():
    w = W._Words(5489)
    first = int(w._bits.random_raw(1)[0])
    assert first == 3499211612      # std::mt19937 default seed, first output


def test_depth_limit_holds():
    spec = W.random_tree(11, 1024)
    depth, peak = 0, 0
    # postfix: primitives push depth 1 subtrees; track the tree depth via a stack of depths
    stack = []
    i = 0
    while i < spec.size:
        op = int(spec[i])
        if op <= W.CONINDER:
            stack.append(1)
        elif op in (W.UNION, W.DIFF, W.INTER, W.BLEND_UNION, W.BLEND_DIFF, W.BLEND_INTER):
            r, l = stack.pop(), stack.pop()
            stack.append(1 + max(l, r))
        i += 1 + W.ARITY[op]
    assert len(stack) == 1 and stack[0] <= 12


def test_export_grid_sizes():
    assert W.export_grid(resolution=128).sx == 130
    assert W.export_grid(resolution=512).corners == 515 ** 3
    assert W.export_grid(resolution=1024).sx == 1026

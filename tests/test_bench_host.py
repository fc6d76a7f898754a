"""Host-side helpers of bench.py that shape what the bench line reports
(no GPU): the staged column variant named in the roofline, the tuning the
persistent ensemble kernel carries, and the algorithmic words per point."""
import bench


def test_column_variant_follows_the_tuning():
    assert bench.column_variant("k_sound_column_tm", [32, 760, 1, 8]) == "k_sound_column_tw12"
    assert bench.column_variant("k_sound_column_tm", [32, 32 | 256 | 24]) == "k_sound_column_tw16"
    assert bench.column_variant("k_sound_column_tm", [32, 56, 1]) == "k_sound_column_tm"
    assert bench.column_variant("k_waf_vertical", [32, 760, 1, 8]) == "k_waf_vertical"
    # every staged variant the bench can name has its ncu traffic and
    # FP64-pipe figures, except the 16-warp kernel the autotuner has not
    # picked on the benchmarked grid
    for v in ("k_sound_column_tm", "k_sound_column_tw12"):
        assert v in bench.NCU_TRAFFIC and v in bench.NCU_FP64_PIPE


def test_persistent_tuning_drops_what_the_persistent_kernel_lacks():
    # horizontal strips -> tiles, ten vertical fields -> one, the staged
    # column solve and the two-level strips -> off, k-marching momentum
    # without strips -> off; the rest kept
    assert bench.persistent_tuning([32, 760, 10, 8]) == [4, 760 & ~(32 | 512), 1]
    assert bench.persistent_tuning([2, 4 | 1, 2]) == [2, 1, 2]
    assert bench.persistent_tuning([8, 24, 1]) == [8, 24, 1]


def test_algorithmic_words_cover_the_profiled_kinds():
    for k in ("k_prediag", "k_sound_divdamp", "k_sound_column_tm", "k_sound_momentum", "k_waf_vertical",
              "k_waf_horizontal", "k_stag_from_x", "k_postdiag"):
        assert bench.ALG_WORDS[k] > 0, k
    assert bench.B_ALG_WORDS == 364

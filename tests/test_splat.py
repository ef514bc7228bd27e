"""Splatmap, CPU side: the demo's rules, argument checks without a device,
and known answers of the oracle restatement
(SuperDemo+/Script/STPSplatmapGenerator.cu, STPTextureSplatRuleWrapper.cu)."""
import ctypes as C

import numpy as np
import pytest

# SuperDemo+/Script/STPBiomeSplatRule.tdl, regions in the script's texture order
# [redrock 0, grass 1, mossrock 2, sand 3, soil 4, darkrock 5]
DEMO_ALTITUDE = [(0, 1.0, 4), (1, 0.5, 3), (1, 0.72, 2), (1, 1.0, 1)]
DEMO_GRADIENT = [(0, 0.0, 0.2, 0.0, 0.27, 3), (1, 0.4, 0.65, 0.58, 0.8, 5), (1, 0.625, 1.0, 0.65, 1.0, 0)]


def test_demo_rules_from_the_library(stpgb):
    alt, gra = stpgb.splat_rules_demo()
    assert [(r.Sample, round(r.UpperBound, 6), r.RegionIndex) for r in alt] == DEMO_ALTITUDE
    assert [(r.Sample, round(r.minGradient, 6), round(r.maxGradient, 6), round(r.LowerBound, 6),
             round(r.UpperBound, 6), r.RegionIndex) for r in gra] == DEMO_GRADIENT


def test_generator_rejects_bad_rules_without_gpu(stpgb):
    s = stpgb.SimplexSetting(42, 8, 0.2181661565)
    with pytest.raises(stpgb.STPNumericDomainError):
        stpgb.STPSplatmapGenerator(DEMO_ALTITUDE, [(0, 0.5, 0.2, 0.0, 1.0, 1)], s, (64, 64))
    with pytest.raises(stpgb.STPNumericDomainError):
        stpgb.STPSplatmapGenerator(DEMO_ALTITUDE, DEMO_GRADIENT, s, (0, 64))
    with pytest.raises(stpgb.STPInvalidEnvironment):
        stpgb.STPSplatmapGenerator(DEMO_ALTITUDE, DEMO_GRADIENT, stpgb.SimplexSetting(1, 0, 0.0), (64, 64))


def test_rule_tables_follow_the_database_order():
    from oracle.oracle import splat_rule_tables
    alt = [(5, 0.9, 1), (2, 0.7, 2), (5, 0.3, 3), (2, 0.1, 4)]
    gra = [(5, 0.0, 1.0, 0.0, 1.0, 7), (2, 0.1, 0.2, 0.0, 1.0, 8), (5, 0.2, 0.3, 0.0, 1.0, 9)]
    d, reg, an, gn = splat_rule_tables(alt, gra)
    assert d.tolist() == [2, 5]
    assert an["RegionIndex"].tolist() == [4, 2, 3, 1] and gn["RegionIndex"].tolist() == [8, 7, 9]
    assert reg.tolist() == [(0, 2, 0, 1), (2, 2, 1, 2)]


def test_oracle_flat_terrain_known_answers(oracle, stpgb):
    """A flat map has slope factor 0 everywhere: sample 0 below altitude 0.27 is sand (gradient rule),
    above it soil (altitude rule); sample 1 follows the altitude ladder; a sample above every
    dictionary entry has no region (255)."""
    perm, grad = stpgb.permutation_generate(42, 8, 0.2181661565)
    S = 32
    for level, sample, want in ((0.05, 0, 3), (0.9, 0, 4), (0.3, 1, 3), (0.95, 1, 1), (0.5, 9, 255)):
        hm = np.full((S, S), int(round(level * 65535)), np.uint16)
        bm = np.full((S, S), sample, np.uint16)
        out, slope, alt = oracle.splatmap(bm, hm, [(0, 0, 0.0, 0.0)], (S, S), DEMO_ALTITUDE, DEMO_GRADIENT, perm,
                                          grad)
        assert np.all(np.abs(slope) <= 1e-6)
        assert np.all((alt >= level - 1e-6) & (alt <= level + 0.15 + 1e-6))
        if want == 3 and sample == 1:
            want_map = np.where(alt <= 0.5, 3, np.where(alt <= 0.72, 2, 1))
            assert np.array_equal(out, want_map)
        else:
            assert np.all(out == want), (level, sample, np.unique(out))

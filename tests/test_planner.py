"""The batch planner's work-item sizing (host logic, no device work),
through the testing entry point rfmf_debug_plan_items: on the item times
per scheduler level measured on GB300 for the bench's two graphs (50x60
torus and ER n = 2000 d = 19, 1024 one-warp chains each, 150 resident
CTAs of up to 16 chains), it must pick the sizes that were fastest when
forced: 16 torus / 12 ER chains per item at P = 128 (11.06 us per sweep
against 12.2-12.4 for every other fitting split) and 12 / 16 at P = 1
(3.74 against 4.52).  When even the largest items need more than one round
of the CTAs, it minimises the queue's longest-first list schedule."""


def _levels(l3, l4):
    # levels 1..4 of a 16-chain one-warp CTA; 1 and 2 only need to be
    # cheaper than 3 (they never fit the slots here)
    return [0.5 * l3, 0.75 * l3, l3, l4]


def test_phase_128_drops_the_dense_graph_to_level_three(rfmf):
    kg = rfmf.debug_plan_items([1024, 1024], 16, 1,
                               [_levels(6.2, 6.5), _levels(11.06, 12.3)], 150)
    assert kg == [16, 12]


def test_phase_1_drops_the_larger_graph_to_level_three(rfmf):
    kg = rfmf.debug_plan_items([1024, 1024], 16, 1,
                               [_levels(3.74, 4.53), _levels(3.2, 3.47)], 150)
    assert kg == [12, 16]


def test_items_stay_within_the_slots(rfmf):
    # equal graphs: both at level 3 would need 172 items > 150 slots, so one
    # of them stays at level 4, and then the makespan is level 4's whatever
    # the other does: both keep full items (fewest CTAs)
    kg = rfmf.debug_plan_items([1024, 1024], 16, 1, [_levels(4.0, 4.5)] * 2, 150)
    assert kg == [16, 16]
    # one graph alone with room for level 3
    kg = rfmf.debug_plan_items([1024, 512], 16, 1, [_levels(4.0, 4.5)] * 2, 150)
    assert kg == [12, 12]


def test_level_boundaries_follow_warps_per_chain(rfmf):
    # two-warp chains: 8 per CTA, levels of 2 chains; the largest size of a
    # level is what the planner offers, so sizes are even
    kg = rfmf.debug_plan_items([300, 300], 8, 2,
                               [[1.0, 2.0, 3.0, 4.0], [1.0, 2.0, 3.0, 4.0]], 400)
    assert all(k % 2 == 0 for k in kg)
    assert kg == [2, 2]


def test_more_than_one_round_minimises_the_list_schedule(rfmf):
    # 768 four-warp chains of three large sparse graphs on 152 CTAs of at
    # most four chains (levels 1..4 = 1..4 chains): the largest items need
    # 192 > 152 slots.  Items of 6.8 / 4.2 / 2.94 us per sweep at level 4
    # (scaled (L + 3) / 7 below) leave 16 cheap items for a second round on
    # the tree's slots (makespan 7.14); three-chain tree items shorten the
    # schedule to the torus items' 6.8, which bounds it.
    lv = lambda t: [t * (L + 3) / 7 for L in (1, 2, 3, 4)]
    kg = rfmf.debug_plan_items([256, 256, 256], 4, 4, [lv(6.8), lv(4.2), lv(2.94)], 152)
    assert kg == [4, 3, 4], kg
    # deep queues: smaller items cost more per chain, so full ones stay
    kg = rfmf.debug_plan_items([5000, 5000], 16, 1, [_levels(1.0, 1.2)] * 2, 100)
    assert kg == [16, 16], kg


def test_one_graph_past_one_round_drops_a_level(rfmf):
    # 3000 one-warp chains of one graph on 152 CTAs of 16: full items take
    # two rounds (188 items); twelve-chain items (level 3, 250 items) also
    # take two, each round 6/7 as long
    kg = rfmf.debug_plan_items([3000], 16, 1, [_levels(6.0, 7.0)], 152)
    assert kg == [12], kg

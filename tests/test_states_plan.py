"""Internal states and reactions in the plan compiler (CPU).

`state : <name> : mon | valence | alphabulk | chi_<X>` keys give a segment
states (State::CheckInput, state.cpp:37-106); `reaction : <name> : equation
| pK | K` keys fix their bulk fractions (Reaction::CheckInput, reaction.cpp:
37-145).  The compiler solves the bulk equilibrium the way the reference's
WEAK pre-iteration does (Solve_scf::Solve, solve_scf.cpp:562-603), builds χ
between the interaction species (segments without states, then states;
system.cpp:1775-1915) and the iteration list with ItStateList after
ItMonList.  The golden fixtures states_* pin the resulting solves to the
reference's own runs (test_oracle_golden); here: the bulk fractions against
values the reference printed, χ defaults, the iteration list, and refusals."""
import pytest

from namics_gb300 import NamicsError, Plan

BASE = """lat : flat : n_layers : 30
lat : flat : lattice_type : simple_cubic
lat : flat : geometry : planar
lat : flat : gradients : 1
lat : flat : lowerbound : surface
lat : flat : bondlength : 3e-10
mon : S : freedom : frozen
mon : S : frozen_range : lowerbound
mon : W : freedom : free
mon : A : freedom : free
mon : Na : freedom : free
mon : Cl : freedom : free
mon : Na : valence : 1
mon : Cl : valence : -1
mon : A : valence : -1
mon : A : chi_S : -1
state : AH : valence : 0
state : AH : mon : A
state : AM : valence : -1
state : AM : mon : A
state : H3O : valence : 1
state : H2O : valence : 0
state : OH : valence : -1
state : H3O : mon : W
state : H2O : mon : W
state : OH : mon : W
reaction : weak : equation : 1(AH) + 1(H2O) = 1(AM) + 1(H3O)
reaction : weak : pK : 7
reaction : auto : equation : 2(H2O) = 1(OH) + 1(H3O)
reaction : auto : pK : 14
state : H3O : alphabulk : {h3o}
mol : water : composition : (W)1
mol : water : freedom : solvent
mol : pol : composition : (A)20
mol : pol : freedom : restricted
mol : pol : theta : 1
mol : Na : composition : (Na)1
mol : Na : freedom : neutralizer
mol : Cl : composition : (Cl)1
mol : Cl : freedom : free
mol : Cl : phibulk : 0.01
"""

# the reference's own .kal output (%.16e) for these inputs: AH, AM, H3O, H2O, OH
REF = {
    "1e-7": [5.0000005000000503e-01, 4.9999994999999497e-01, 9.9999999999999995e-08,
             9.9999979999999999e-01, 1.0000000000000001e-07],   # guesses kept (no Newton step)
    "1e-5": [9.9009910794040767e-01, 9.9008920595923637e-03, 1.0000000000000001e-05,
             9.9998999900001995e-01, 9.9997999809763420e-10],   # Newton steps to the root
    "1e-3": [9.9990010997901413e-01, 9.9890020985905688e-05, 1.0000000000000000e-03,
             9.9899999999001998e-01, 9.9800099998006252e-12],
}


@pytest.mark.parametrize("h3o", sorted(REF))
def test_bulk_fractions_are_the_references(h3o):
    p = Plan(BASE.format(h3o=h3o))
    assert p.state_names == ["AH", "AM", "H3O", "H2O", "OH"]
    for got, want in zip(p.state_alphabulk, REF[h3o]):
        assert abs(got - want) <= 1e-11 * want, (got, want)


def test_species_and_iteration_list():
    p = Plan(BASE.format(h3o="1e-7"))
    c = p.c
    ns, nst = c.n_seg, c.n_state
    assert (ns, nst, c.n_sp) == (5, 5, 10)
    segs = p.seg_names
    assert [segs[c.state_seg[j]] for j in range(nst)] == ["A", "A", "W", "W", "W"]
    assert [c.seg_nstate[i] for i in range(ns)] == [0, 3, 2, 0, 0]  # S, W, A, Na, Cl
    # a segment with states carries no valence of its own; its states do
    assert c.seg_valence[segs.index("A")] == 0
    assert [c.state_valence[j] for j in range(nst)] == [0, -1, 1, 0, -1]
    assert c.charged == 1
    chi = lambda a, b: c.chi_sp[a * c.n_sp + b]
    # states take their mon's χ where none is given: AH, AM with S at -1
    assert chi(ns + 0, segs.index("S")) == -1 and chi(segs.index("S"), ns + 1) == -1
    assert chi(ns + 2, segs.index("S")) == 0
    # ItMonList: Na (Cl has Na's χ row); ItStateList: AH (AM has its row),
    # the water states share Na's block (all-zero rows)
    assert p.it_names == ["Na", "AH"]
    assert [c.state_it[j] for j in range(nst)] == [1, 1, 0, 0, 0]
    assert c.seg_it[segs.index("A")] == -1 and c.seg_it[segs.index("W")] == -1
    # the bulk charge of the molecules: Σ α_bulk·valence of the states
    assert abs(c.mols[1].charge - (-p.state_alphabulk[1])) < 1e-15
    assert abs(c.mols[0].charge - (p.state_alphabulk[2] - p.state_alphabulk[4])) < 1e-15
    assert c.iv == 3 * c.M


def test_state_chi_keys():
    t = BASE.format(h3o="1e-7") + "state : AH : chi_H2O : 0.8\nmon : Na : chi_AM : 0.2\n"
    p = Plan(t)
    c = p.c
    ns = c.n_seg
    chi = lambda a, b: c.chi_sp[a * c.n_sp + b]
    assert chi(ns + 0, ns + 3) == 0.8 and chi(ns + 3, ns + 0) == 0.8
    na = p.seg_names.index("Na")
    assert chi(na, ns + 1) == 0.2 and chi(ns + 1, na) == 0.2
    # every state row differs now: AH, AM and H2O get blocks of their own
    assert p.it_names == ["Na", "Cl", "AH", "AM", "H2O"]


@pytest.mark.parametrize("edit", [
    lambda t: t.replace("state : OH : mon : W\n", "").replace("state : OH : valence : -1\n", "")
              .replace("2(H2O) = 1(OH) + 1(H3O)", "2(H2O) = 1(H3O) + 1(H3O)"),            # not balanced
    lambda t: t.replace("reaction : auto : pK : 14", "reaction : auto : pK : 14\nstate : OH : valence : -2"),
    lambda t: t.replace("state : H3O : alphabulk : 1e-7\n", ""),                        # too few fixed
    lambda t: t + "state : AH : alphabulk : 0.5\n",                                      # too many fixed
    lambda t: t.replace("1(AH) + 1(H2O)", "1(AX) + 1(H2O)"),                              # unknown state
    lambda t: t.replace("reaction : weak : pK : 7\n", ""),                               # no pK / K
    lambda t: t + "mon : A : chi_AH : 0.5\n",                                            # χ mon–own state
    lambda t: t.replace("mol : pol : theta : 1", "mol : pol : theta : 1\nmol : pol : Markov : 2\n"
                        "mol : pol : k_stiff : 1"),
    lambda t: t.replace("state : AH : mon : A", "state : AH : mon : S"),                 # frozen mon
    lambda t: t.replace("state : AH : mon : A", "state : AH : mon : Q"),                 # no such mon
], ids=["unbalanced", "not_neutral", "too_few_fixed", "too_many_fixed", "unknown_state", "no_pK",
        "chi_own_state", "markov2", "frozen_mon", "no_mon"])
def test_refused(edit):
    with pytest.raises(NamicsError):
        Plan(edit(BASE.format(h3o="1e-7")))


def test_a_lone_state_and_reactions_without_states_are_refused():
    lone = BASE.format(h3o="1e-7")
    lone = "\n".join(ln for ln in lone.splitlines()
                     if not ln.startswith(("state", "reaction")) or ln.startswith("state : AH")) + "\n"
    with pytest.raises(NamicsError):
        Plan(lone)
    none = "\n".join(ln for ln in BASE.format(h3o="1e-7").splitlines() if not ln.startswith("state")) + "\n"
    with pytest.raises(NamicsError):
        Plan(none)


def test_search_with_states_is_refused():
    t = BASE.format(h3o="1e-7") + "var : mol-pol : search : theta\nvar : sys-noname : free_energy : -5\n"
    with pytest.raises(NamicsError):
        Plan(t)


def test_batched_solver_refuses_states():
    from namics_gb300 import NM_FP64, Batch
    p = Plan(BASE.format(h3o="1e-7"))
    with pytest.raises(NamicsError):
        Batch([p], NM_FP64)


def test_K_is_ten_to_the_minus_pK():
    """`reaction : <name> : K` instead of pK (reaction.cpp:60-68): pK = -log10(K)."""
    a = Plan(BASE.format(h3o="1e-5"))
    b = Plan(BASE.format(h3o="1e-5").replace("reaction : weak : pK : 7", "reaction : weak : K : 1e-7"))
    for x, y in zip(a.state_alphabulk, b.state_alphabulk):
        assert abs(x - y) <= 1e-12 * x


def test_state_scan_keys():
    """`var : state-<name> : scan : alphabulk` on a fixed state, and a reaction's
    pK scan; a scan of a state the reactions set is refused."""
    t = BASE.format(h3o="1e-7")
    p = Plan(t + "var : state-H3O : scan : alphabulk\nvar : state-H3O : scale : exponential\n"
                 "var : state-H3O : end_value : 1e-4\nvar : state-H3O : steps : 2\n")
    assert p.c.scan_state == p.state_names.index("H3O") and p.c.scan_n == 6
    v = p.scan_values()
    assert v[0] == pytest.approx(1e-7) and v[-1] == pytest.approx(1e-4) and v[2] == pytest.approx(1e-6)
    q = Plan(t + "var : reaction-weak : scan : pK\nvar : reaction-weak : step : 0.5\n"
                 "var : reaction-weak : end_value : 8\n")
    assert q.c.scan_reaction == 0 and q.scan_values() == [7.0, 7.5, 8.0]
    with pytest.raises(NamicsError):  # AM's fraction follows from the reactions
        Plan(t + "var : state-AM : scan : alphabulk\nvar : state-AM : step : 0.1\nvar : state-AM : end_value : 0.9\n")
    with pytest.raises(NamicsError):  # a pK scan is linear
        Plan(t + "var : reaction-weak : scan : pK\nvar : reaction-weak : scale : exponential\n"
                 "var : reaction-weak : end_value : 8\n")


@pytest.mark.parametrize("name", ["scan_states_h3o", "scan_states_pk"])
def test_bulk_equilibrium_follows_the_reference_scan(name):
    """nm_plan_state_bulk with the previous step's bulk volume fractions
    gives the reference's bulk fractions of the next scan step: the oracle
    solves each step with the reference's own fractions, its species' bulk
    fractions then feed the next step's equilibrium (Reaction::pKeff reads
    them, with the reference's term-position indexing of the states)."""
    import sys
    from pathlib import Path
    import numpy as np
    from conftest import load_golden
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    from orc import Oracle
    g = load_golden(name)
    plan = Plan(g["input"])
    c = plan.c
    orc = Oracle(plan)
    names = [f"mon_{plan.seg_names[c.state_seg[j]]}_alphabulk_{st}" for j, st in enumerate(plan.state_names)]
    values = plan.scan_values()
    x = np.array(g["x"])
    # step 0: no previous solve, pK_eff = pK, the plan's fractions
    ab0, _ = plan.state_bulk()
    assert np.allclose(ab0, plan.state_alphabulk, rtol=1e-15, atol=0)
    fixed = np.array(plan.state_alphabulk)
    pk = None
    for k, row in enumerate(g["rows"]):
        if k > 0:
            if c.scan_state >= 0:
                fixed[c.scan_state] = values[k]
            else:  # the input's reactions: weak (scanned), then auto at pK 14
                assert c.scan_reaction == 0
                pk = [values[k], 14.0]
            ab, _ = plan.state_bulk(fixed_ab=fixed, pK=pk, sp_phibulk=orc.species_phibulk())
            ref = np.array([row[n] for n in names])
            assert np.max(np.abs(ab - ref) / ref) < 1e-6, (k, ab, ref)
        orc.set_states([row[n] for n in names])
        rc, x, _, res = orc.solve(x)
        assert rc == 0

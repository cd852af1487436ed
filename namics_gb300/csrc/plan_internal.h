// Owning storage behind the public nm_plan view.
#pragma once
#include <functional>
#include <string>
#include <vector>

#include "../../include/namics_gb300.h"

namespace nm {

void set_error(const std::string& msg);

struct MolBuild {
    nm_molecule mol{};
    std::vector<nm_block> blocks;
    std::vector<int> child_index;
    std::vector<int> molmon;
    std::vector<double> fraction;
    int n_store = 0;
    bool is_dendrimer = false;
};

// One reaction: the states of its equation in written order and their
// stoichiometric numbers, negative on the left-hand side (Reaction::
// CheckInput, reaction.cpp:37-145).
struct ReactionDef {
    std::string name;
    double pK = 0;
    std::vector<int> sto, state;
};

// `plan` must stay the first member: nm_plan* and PlanHolder* are converted
// into each other.
struct PlanHolder {
    nm_plan plan{};
    std::vector<double> L, lm1, l0, lp1;
    std::vector<int> ksam;
    std::vector<std::string> seg_names;
    std::vector<const char*> seg_name_ptrs;
    std::vector<int> seg_freedom, seg_it, it_seg;
    std::vector<double> seg_mask, seg_gmask, seg_phi_frozen, chi, seg_valence, seg_epsilon;
    std::vector<MolBuild> mb;
    std::vector<nm_molecule> mols;
    // internal states and reactions (n_state = 0 when the input has none)
    std::vector<std::string> state_names;
    std::vector<const char*> state_name_ptrs;
    std::vector<int> state_seg, state_it, seg_nstate, it_sp;
    std::vector<double> state_valence, state_alphabulk, chi_sp;
    std::vector<ReactionDef> reactions;
    std::vector<char> state_fixed;     // alphabulk given in the input
    std::vector<double> state_ab_in;   // the input's alphabulk (-1 where none)
    std::vector<double> mol_nmon;      // per molecule and molmon: segments of that type
    std::vector<std::string> mol_names;
    std::vector<const char*> mol_name_ptrs;
    std::string method_note;
};

// The states' bulk fractions and the molecules' charges of a plan with
// internal states, the fixed states' alphabulk taken from `fixed_ab`
// [n_state] (other entries unused; a `var : state-<name> : scan :
// alphabulk` step, State::UpdateVarInfo, state.cpp:306-318), the
// reactions' pK from `pK` [reactions] (a `var : reaction-<name> : scan :
// pK` step, Reaction::UpdateVarInfo, reaction.cpp:410-425) and their pK_eff
// from the species' bulk volume fractions `sp_phibulk` [n_sp] of the last
// solve (null before any).
int plan_state_bulk(const nm_plan* p, const std::vector<double>& fixed_ab, const std::vector<double>& pK,
                    const double* sp_phibulk, std::vector<double>& alphabulk, std::vector<double>& mol_charge,
                    std::string& err);
// the reactions' pK of the input, in input order
std::vector<double> plan_reaction_pK(const nm_plan* p);
// reaction index by name, or -1
int plan_reaction_index(const nm_plan* p, const std::string& name);

}  // namespace nm

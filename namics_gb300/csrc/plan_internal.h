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
    std::vector<std::string> mol_names;
    std::vector<const char*> mol_name_ptrs;
    std::string method_note;
};

}  // namespace nm

// .pro and .kal output of a device context, in the reference's file layout
// (Output::WriteOutput, output.cpp:385-564; LGrad1/2/3::PutProfiles,
// LGrad1.cpp:228-248, LGrad2.cpp:185-203, LGrad3.cpp:81-100), so tools that
// read the reference's outputs read these.
//
// Items are the `key : name : property` triples of an input's output block.
// The header joins each triple with '_' (the default header separator); a
// .pro row is the site's coordinates then the profile values, interior sites
// only, x outermost; a .kal file is one header line and one line of values
// per call.  Number formats are the reference's: coordinates %e, profiles
// %.20g (1 gradient) or %.20e followed by a tab (2 and 3 gradients), scalars
// %.16e, integers %i.
#include <cstdio>
#include <string>
#include <vector>

#include "ctx_internal.h"

namespace nm {

namespace {

std::string trim(const std::string& s) {
    size_t a = s.find_first_not_of(" \t"), b = s.find_last_not_of(" \t");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// "key : name : prop" -> its three parts
bool split3(const char* item, std::string& key, std::string& name, std::string& prop) {
    std::string s(item ? item : "");
    size_t p1 = s.find(':');
    if (p1 == std::string::npos) return false;
    size_t p2 = s.find(':', p1 + 1);
    if (p2 == std::string::npos) return false;
    key = trim(s.substr(0, p1));
    name = trim(s.substr(p1 + 1, p2 - p1 - 1));
    prop = trim(s.substr(p2 + 1));
    return !key.empty() && !name.empty() && !prop.empty();
}

int seg_index(const nm_plan* p, const std::string& n) {
    for (int i = 0; i < p->n_seg; i++)
        if (n == p->seg_name[i]) return i;
    return -1;
}
// state j of segment k named `st`, or -1
int state_of(const nm_plan* p, int k, const std::string& st) {
    for (int j = 0; j < p->n_state; j++)
        if (p->state_seg[j] == k && st == p->state_name[j]) return j;
    return -1;
}
int mol_index(const nm_plan* p, const std::string& n) {
    for (int m = 0; m < p->n_mol; m++)
        if (p->mol_name && n == p->mol_name[m]) return m;
    return -1;
}

}  // namespace

}  // namespace nm

extern "C" {

int nm_write_pro(nm_ctx* ctx, const char* path, const char* const* items, int n_items) {
    using namespace nm;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !path || (n_items > 0 && !items)) { set_error("nm_write_pro: bad argument"); return NM_ERR_ARG; }
    if (!c->have_state) { set_error("nm_write_pro: no residual evaluated yet"); return NM_ERR_ARG; }
    const nm_plan* p = c->plan;
    const size_t M = p->M;
    // the fields the items draw from, fetched once each
    std::vector<std::vector<double>> field(12);
    auto get = [&](int which, size_t n) -> int {
        if (field[which].empty()) {
            field[which].resize(n);
            int rc = nm_get_field(ctx, which, field[which].data());
            if (rc) return rc;
        }
        return NM_OK;
    };
    std::vector<const double*> cols;
    std::vector<std::string> heads;
    for (int i = 0; i < n_items; i++) {
        std::string key, name, prop;
        if (!split3(items[i], key, name, prop)) { set_error(std::string("nm_write_pro: not a 'key : name : property' item: ") + (items[i] ? items[i] : "")); return NM_ERR_ARG; }
        const double* col = nullptr;
        int rc = NM_OK;
        if (key == "mon") {
            int k = seg_index(p, name);
            if (k >= 0 && prop == "phi") { rc = get(0, p->n_seg * M); col = field[0].data() + k * M; }
            else if (k >= 0 && prop == "G1") { rc = get(1, p->n_seg * M); col = field[1].data() + k * M; }
            else if (k >= 0 && p->n_state > 0) {
                // a state's φ, α or u (Segment::GetPointer, segment.cpp:1896-1910).
                // The reference's file holds zeros in the φ column of a mon's
                // first state (its profile index 2 is the 3-D φ[z] average,
                // reached for 1 and 2 gradients too); this writes the values.
                const size_t dash = prop.find('-');
                const std::string what = dash == std::string::npos ? "" : prop.substr(0, dash);
                const int j = dash == std::string::npos ? -1 : state_of(p, k, prop.substr(dash + 1));
                const int which = what == "phi" ? 9 : what == "alpha" ? 10 : what == "u" ? 11 : -1;
                if (j >= 0 && which > 0) { rc = get(which, (size_t)p->n_state * M); col = field[which].data() + j * M; }
            }
        } else if (key == "mol") {
            int m = mol_index(p, name);
            if (m >= 0 && prop == "phi") { rc = get(4, p->n_mol * M); col = field[4].data() + m * M; }
        } else if (key == "sys") {
            if (prop == "alpha") { rc = get(2, M); col = field[2].data(); }
            else if (prop == "phitot") { rc = get(3, M); col = field[3].data(); }
            else if (p->charged && prop == "psi") { rc = get(6, M); col = field[6].data(); }
            else if (p->charged && prop == "q") { rc = get(7, M); col = field[7].data(); }
            else if (p->charged && prop == "eps") { rc = get(8, M); col = field[8].data(); }
        }
        if (rc) return rc;
        if (!col) { set_error("nm_write_pro: not a profile of this problem: " + key + " : " + name + " : " + prop); return NM_ERR_ARG; }
        cols.push_back(col);
        heads.push_back(key + "_" + name + "_" + prop);
    }
    FILE* fp = std::fopen(path, "w");
    if (!fp) { set_error(std::string("nm_write_pro: cannot open ") + path); return NM_ERR_ARG; }
    const int g = p->gradients, n = (int)cols.size();
    std::fputs(g == 1 ? "x\t" : (g == 2 ? "x\ty\t" : "x\ty\tz\t"), fp);
    for (int i = 0; i < n; i++) std::fprintf(fp, i < n - 1 ? "%s\t" : "%s", heads[i].c_str());
    std::fputs("\n", fp);
    const double off = p->offset_first_layer, one = 1.0;
    if (g == 1) {
        for (int x = 1; x <= p->MX; x++) {
            std::fprintf(fp, "%e\t", off / 1 + 1.0 * (x - 1 + 1) / 1 - 0.5 / 1);
            for (int i = 0; i < n; i++) std::fprintf(fp, i < n - 1 ? "%.20g\t" : "%.20g", cols[i][x]);
            std::fputs("\n", fp);
        }
    } else if (g == 2) {
        for (int x = 1; x <= p->MX; x++)
            for (int y = 1; y <= p->MY; y++) {
                std::fprintf(fp, "%e\t%e\t", off / 1 + one * (x - 1 + 1) / 1 - 0.5 / 1, one * (y - 1 + 1) / 1 - 0.5 / 1);
                for (int i = 0; i < n; i++) std::fprintf(fp, "%.20e\t", cols[i][x * p->JX + y]);
                std::fputs("\n", fp);
            }
    } else {
        for (int x = 1; x <= p->MX; x++)
            for (int y = 1; y <= p->MY; y++)
                for (int z = 1; z <= p->MZ; z++) {
                    std::fprintf(fp, "%e\t%e\t%e\t", one * (x - 1 + 1) / 1 - 0.5 / 1, one * (y - 1 + 1) / 1 - 0.5 / 1,
                                 one * (z - 1 + 1) / 1 - 0.5 / 1);
                    for (int i = 0; i < n; i++) std::fprintf(fp, "%.20e\t", cols[i][x * p->JX + y * p->JY + z]);
                    std::fputs("\n", fp);
                }
    }
    if (std::fclose(fp) != 0) { set_error(std::string("nm_write_pro: write failed: ") + path); return NM_ERR_ARG; }
    return NM_OK;
}

int nm_write_kal(nm_ctx* ctx, const char* path, const char* const* items, int n_items, const nm_solve_result* res,
                 int append) {
    using namespace nm;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !path || (n_items > 0 && !items)) { set_error("nm_write_kal: bad argument"); return NM_ERR_ARG; }
    if (!c->have_state) { set_error("nm_write_kal: no residual evaluated yet"); return NM_ERR_ARG; }
    const nm_plan* p = c->plan;
    double F = 0, Om = 0;
    std::vector<double> mu(p->n_mol);
    bool have_fe = false;
    std::vector<double> molphi;
    struct Val { bool is_int; int i; double d; };
    std::vector<Val> vals;
    std::vector<std::string> heads;
    for (int k = 0; k < n_items; k++) {
        std::string key, name, prop;
        if (!split3(items[k], key, name, prop)) { set_error(std::string("nm_write_kal: not a 'key : name : property' item: ") + (items[k] ? items[k] : "")); return NM_ERR_ARG; }
        Val v{false, 0, 0.0};
        bool ok = false;
        auto fe = [&]() -> int {
            if (!have_fe) { int rc = c->free_energy(&F, &Om, mu.data()); if (rc) return rc; have_fe = true; }
            return NM_OK;
        };
        if (key == "sys" && (prop == "free_energy" || prop == "grand_potential")) {
            int rc = fe();
            if (rc) return rc;
            v.d = prop == "free_energy" ? F : Om;
            ok = true;
        } else if (key == "newton" && res && (prop == "residual" || prop == "iterations")) {
            if (prop == "residual") v.d = res->residual;
            else { v.is_int = true; v.i = res->iterations; }
            ok = true;
        } else if (key == "mon" && p->n_state > 0 && seg_index(p, name) >= 0) {
            // a state's scalars (Segment::PushOutput, segment.cpp:1820-1830):
            // alphabulk_, valence_, phibulk_ (φ_bulk of the mon × α_bulk),
            // theta_ (Σ over the interior of L·φ_state) and theta_exc_
            // (θ − volume·φ_bulk)
            const int k = seg_index(p, name);
            static const char* const kinds[] = {"alphabulk_", "valence_", "phibulk_", "theta_exc_", "theta_"};
            for (const char* kd : kinds) {
                const std::string pre(kd);
                if (prop.compare(0, pre.size(), pre) != 0) continue;
                const int j = state_of(p, k, prop.substr(pre.size()));
                if (j < 0) break;
                if (pre == "alphabulk_") v.d = c->st.ab[j];  // the context's (a scan may have moved them)
                else if (pre == "valence_") v.d = p->state_valence[j];
                else {
                    std::vector<double> spb((size_t)c->nsp);
                    cudaError_t e = cudaMemcpyAsync(spb.data(), c->d_seg_phibulk, sizeof(double) * spb.size(),
                                                    cudaMemcpyDeviceToHost, c->stream);
                    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
                    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
                    const double pb = spb[(size_t)p->n_seg + j];
                    if (pre == "phibulk_") v.d = pb;
                    else {
                        const size_t M = p->M;
                        std::vector<double> ph((size_t)p->n_state * M);
                        int rc = nm_get_field(ctx, 9, ph.data());
                        if (rc) return rc;
                        const bool w = p->gradients < 3 && p->geometry != NM_PLANAR;
                        double sum = 0;
                        for (int x = 1; x <= p->MX; x++)
                            for (int y = (p->gradients > 1 ? 1 : 0); y <= (p->gradients > 1 ? p->MY : 0); y++)
                                for (int z = (p->gradients > 2 ? 1 : 0); z <= (p->gradients > 2 ? p->MZ : 0); z++) {
                                    const size_t s = (size_t)x * p->JX + (size_t)y * p->JY + z;
                                    sum += w ? ph[(size_t)j * M + s] * p->L[s] : ph[(size_t)j * M + s];
                                }
                        v.d = pre == "theta_" ? sum : sum - p->volume * pb;
                    }
                }
                ok = true;
                break;
            }
        } else if (key == "reaction" && prop == "pK" && p->n_state > 0) {
            // the reaction's pK in force (Reaction::PushOutput, reaction.cpp:188-201)
            const int r = plan_reaction_index(p, name);
            if (r >= 0) { v.d = c->st_pK[r]; ok = true; }
        } else if (key == "mol") {
            int m = mol_index(p, name);
            if (m >= 0) {
                double GN, n, th, pb;
                if (prop == "Mu") {
                    int rc = fe();
                    if (rc) return rc;
                    v.d = mu[m];
                    ok = true;
                } else if (prop == "theta") {
                    // the amount in the system, Σ L·φ over the interior, as the
                    // reference computes it for its output (molecule.cpp:2006-2009)
                    const size_t M = p->M;
                    if (molphi.empty()) {
                        molphi.resize((size_t)p->n_mol * M);
                        int rc = nm_get_field(ctx, 4, molphi.data());
                        if (rc) return rc;
                    }
                    const bool w = p->gradients < 3 && p->geometry != NM_PLANAR;
                    double sum = 0;
                    const double* ph = molphi.data() + (size_t)m * M;
                    for (int x = 1; x <= p->MX; x++)
                        for (int y = (p->gradients > 1 ? 1 : 0); y <= (p->gradients > 1 ? p->MY : 0); y++)
                            for (int z = (p->gradients > 2 ? 1 : 0); z <= (p->gradients > 2 ? p->MZ : 0); z++) {
                                const size_t s = (size_t)x * p->JX + (size_t)y * p->JY + z;
                                sum += w ? ph[s] * p->L[s] : ph[s];
                            }
                    v.d = sum;
                    ok = true;
                } else if (prop == "GN" || prop == "n" || prop == "phibulk") {
                    int rc = nm_get_molecule(ctx, m, &GN, &n, &th, &pb);
                    if (rc) return rc;
                    v.d = prop == "GN" ? GN : prop == "n" ? n : pb;
                    ok = true;
                }
            }
        }
        if (!ok) { set_error("nm_write_kal: not a scalar of this problem: " + key + " : " + name + " : " + prop); return NM_ERR_ARG; }
        vals.push_back(v);
        heads.push_back(key + "_" + name + "_" + prop);
    }
    FILE* fp = std::fopen(path, append ? "a" : "w");
    if (!fp) { set_error(std::string("nm_write_kal: cannot open ") + path); return NM_ERR_ARG; }
    const int n = (int)vals.size();
    if (!append) {
        for (int k = 0; k < n; k++) std::fprintf(fp, k < n - 1 ? "%s\t" : "%s", heads[k].c_str());
        std::fputs("\n", fp);
    }
    for (int k = 0; k < n; k++) {
        if (vals[k].is_int) std::fprintf(fp, k < n - 1 ? "%i\t" : "%i", vals[k].i);
        else std::fprintf(fp, k < n - 1 ? "%.16e\t" : "%.16e", vals[k].d);
    }
    std::fputs("\n", fp);
    if (std::fclose(fp) != 0) { set_error(std::string("nm_write_kal: write failed: ") + path); return NM_ERR_ARG; }
    return NM_OK;
}

}  // extern "C"

// Host-side problem compiler: Namics input text -> nm_plan.
//
// Replaces the object construction and the Check/Prepare steps that the
// reference runs before its SCF loop (namics.cpp:165-417; Lattice::CheckInput
// lattice.cpp:267-601, AllocateMemory :79-234; Segment::ParseFreedoms
// segment.cpp:156-792; Molecule::Decomposition molecule.cpp:1282-1779;
// System::CheckChi_values, generate_mask, MakeItsLists system.cpp:190-500).
// Only the key subset an SCF solve of the supported problem classes needs is
// understood; anything else is reported, never silently ignored when it
// would change the result.
#include "plan_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace nm {

thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

namespace {

const double PIE = 3.14159265;  // namics.cpp:49 (the reference's truncated pi)

std::string trim(const std::string& s) {
    size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
}

std::vector<std::string> split(const std::string& s, char c) {
    std::vector<std::string> out;
    std::string cur;
    for (char ch : s) {
        if (ch == c) { out.push_back(cur); cur.clear(); }
        else cur.push_back(ch);
    }
    out.push_back(cur);
    return out;
}

struct Entry {
    std::string cls, name, key, value;
    mutable bool used = false;  // read by the compiler
};

// Keyed view of one `start` block of the input (input.cpp:3-78).
struct InputBlock {
    std::vector<Entry> entries;
    std::vector<std::string> order(const std::string& cls) const {
        std::vector<std::string> names;
        for (auto& e : entries)
            if (e.cls == cls && std::find(names.begin(), names.end(), e.name) == names.end())
                names.push_back(e.name);
        return names;
    }
    bool has(const std::string& cls, const std::string& name, const std::string& key) const {
        bool found = false;
        for (auto& e : entries)
            if (e.cls == cls && e.name == name && e.key == key) { e.used = true; found = true; }
        return found;
    }
    std::string get(const std::string& cls, const std::string& name, const std::string& key,
                    const std::string& dflt = "") const {
        std::string v = dflt;  // last occurrence wins
        for (auto& e : entries)
            if (e.cls == cls && e.name == name && e.key == key) { v = e.value; e.used = true; }
        return v;
    }
};

bool parse_input(const std::string& text, InputBlock& blk) {
    std::istringstream is(text);
    std::string line;
    while (std::getline(is, line)) {
        size_t c = line.find("//");
        if (c != std::string::npos) line = line.substr(0, c);
        line = trim(line);
        if (line.empty()) continue;
        if (line == "start") break;  // first start block only
        std::vector<std::string> p = split(line, ':');
        if (p.size() < 4) {
            set_error("input line not of the form 'class : name : key : value': " + line);
            return false;
        }
        Entry e;
        e.cls = trim(p[0]); e.name = trim(p[1]); e.key = trim(p[2]);
        std::string v = p[3];
        for (size_t i = 4; i < p.size(); i++) v += ":" + p[i];
        e.value = trim(v);
        blk.entries.push_back(e);
    }
    return true;
}

bool to_int(const std::string& s, int& v) {
    char* end = nullptr;
    long r = std::strtol(s.c_str(), &end, 10);
    if (end == s.c_str() || *end != '\0') return false;
    v = (int)r;
    return true;
}

bool to_real(const std::string& s, double& v) {
    char* end = nullptr;
    double r = std::strtod(s.c_str(), &end);
    if (end == s.c_str() || *end != '\0') return false;
    v = r;
    return true;
}

int bc_code(const std::string& s, bool& ok) {
    if (s == "mirror") return NM_BC_MIRROR;
    if (s == "periodic") return NM_BC_PERIODIC;
    if (s == "surface") return NM_BC_SURFACE;
    ok = false;
    return 0;
}

// ---- composition grammar -------------------------------------------------
// A written chain is a list of items: runs `(name)count`, repeated groups
// `((...)...)count` and side chains `[...]` attached to the segment written
// just before the bracket (molecule.cpp:1156-1275, mol_branched.cpp).

struct SegNode {  // one segment of the written molecule
    int seg;
    int parent = -1;               // towards the root
    std::vector<int> children;
};

struct CompParser {
    const std::string& s;
    size_t pos = 0;
    const std::map<std::string, int>& segidx;
    std::string err;
    CompParser(const std::string& s_, const std::map<std::string, int>& m) : s(s_), segidx(m) {}

    bool read_int(int& v) {
        size_t st = pos;
        while (pos < s.size() && isdigit((unsigned char)s[pos])) pos++;
        if (st == pos) return false;
        v = std::atoi(s.substr(st, pos - st).c_str());
        return true;
    }
    // parse a chain until ']' or end; emits a flat token list where
    // side chains are nested vectors.
    struct Item { int seg = -1; int count = 0; std::vector<Item> side; bool is_side = false; };

    bool parse_chain(std::vector<Item>& out, bool inside_bracket) {
        while (pos < s.size()) {
            char c = s[pos];
            if (c == ' ') { pos++; continue; }
            if (c == ']') {
                if (!inside_bracket) { err = "unbalanced ']'"; return false; }
                return true;
            }
            if (c == '[') {
                pos++;
                Item side; side.is_side = true;
                if (!parse_chain(side.side, true)) return false;
                if (pos >= s.size() || s[pos] != ']') { err = "missing ']'"; return false; }
                pos++;
                out.push_back(side);
                continue;
            }
            if (c == '(') {
                // find matching ')'
                int depth = 0; size_t q = pos;
                for (; q < s.size(); q++) {
                    if (s[q] == '(') depth++;
                    else if (s[q] == ')') { depth--; if (depth == 0) break; }
                }
                if (q >= s.size()) { err = "unbalanced '('"; return false; }
                std::string inner = s.substr(pos + 1, q - pos - 1);
                pos = q + 1;
                int cnt;
                if (!read_int(cnt) || cnt < 1) { err = "repeat count expected after ')'"; return false; }
                if (inner.find('(') != std::string::npos || inner.find('[') != std::string::npos) {
                    // repeated group: expand
                    CompParser sub(inner, segidx);
                    std::vector<Item> grp;
                    if (!sub.parse_chain(grp, false)) { err = sub.err; return false; }
                    for (int r = 0; r < cnt; r++) out.insert(out.end(), grp.begin(), grp.end());
                } else {
                    auto it = segidx.find(trim(inner));
                    if (it == segidx.end()) { err = "segment '" + inner + "' in composition is not a mon"; return false; }
                    Item run; run.seg = it->second; run.count = cnt;
                    out.push_back(run);
                }
                continue;
            }
            err = std::string("unexpected character '") + c + "' in composition";
            return false;
        }
        return true;
    }
};

// Emit segment nodes for a parsed chain.  Returns false on grammar errors.
bool emit_chain(const std::vector<CompParser::Item>& items, std::vector<SegNode>& nodes,
                int attach, std::vector<int>& chain_order, std::string& err) {
    int prev = attach;  // segment the next one bonds to
    for (auto& it : items) {
        if (it.is_side) {
            if (prev < 0) { err = "side chain '[' before any segment"; return false; }
            if (!emit_chain(it.side, nodes, prev, chain_order, err)) return false;
            continue;  // the main chain continues from `prev`
        }
        for (int k = 0; k < it.count; k++) {
            SegNode n; n.seg = it.seg;
            nodes.push_back(n);
            int id = (int)nodes.size() - 1;
            chain_order.push_back(id);
            if (prev >= 0) {
                // bond prev -- id (direction fixed later)
                nodes[id].parent = prev;
            }
            prev = id;
        }
    }
    return true;
}

}  // namespace

// Turn an undirected written tree (parent = previous written segment) into a
// rooted tree at `root` and compress it into blocks.
static bool build_blocks_from_tree(std::vector<SegNode>& nodes, int root, PlanHolder& H,
                                   MolBuild& mb, std::string& err) {
    int n = (int)nodes.size();
    std::vector<std::vector<int>> adj(n);
    for (int i = 0; i < n; i++)
        if (nodes[i].parent >= 0) { adj[i].push_back(nodes[i].parent); adj[nodes[i].parent].push_back(i); }
    // BFS from root to orient
    std::vector<int> par(n, -2), order;
    order.reserve(n);
    par[root] = -1; order.push_back(root);
    for (size_t q = 0; q < order.size(); q++) {
        int u = order[q];
        for (int v : adj[u]) if (par[v] == -2) { par[v] = u; order.push_back(v); }
    }
    if ((int)order.size() != n) { err = "composition is not connected"; return false; }
    std::vector<std::vector<int>> ch(n);
    // children in written order (stable): iterate nodes in index order
    for (int i = 0; i < n; i++) if (par[i] >= 0) ch[par[i]].push_back(i);
    // block starts: segment with !=1 children, or whose single child differs in type
    std::vector<int> blk_of(n, -1);
    // build blocks root-ward from each start
    struct TmpBlock { int seg; std::vector<int> segs; int parent_seg; };
    std::vector<TmpBlock> tb;
    for (int i = 0; i < n; i++) {
        bool start = (ch[i].size() != 1) || (nodes[ch[i][0]].seg != nodes[i].seg);
        if (!start) continue;
        TmpBlock b; b.seg = nodes[i].seg;
        int cur = i;
        b.segs.push_back(cur);
        while (true) {
            int p = par[cur];
            if (p < 0) break;
            if (ch[p].size() != 1 || nodes[p].seg != b.seg) break;
            cur = p;
            b.segs.push_back(cur);
        }
        b.parent_seg = par[cur];
        for (int sgi : b.segs) blk_of[sgi] = (int)tb.size();
        tb.push_back(b);
    }
    for (int i = 0; i < n; i++) if (blk_of[i] < 0) { err = "internal: block cover"; return false; }
    int nb = (int)tb.size();
    std::vector<int> bparent(nb, -1);
    std::vector<std::vector<int>> bchildren(nb);
    int broot = blk_of[root];
    for (int b = 0; b < nb; b++) {
        if (tb[b].parent_seg >= 0) {
            int pb = blk_of[tb[b].parent_seg];
            // children must attach at the parent block's first segment
            if (tb[pb].segs.front() != tb[b].parent_seg) { err = "internal: join not at block start"; return false; }
            bparent[b] = pb;
        }
    }
    // children order: by the written index of the child block's top segment
    for (int b = 0; b < nb; b++) if (bparent[b] >= 0) bchildren[bparent[b]].push_back(b);
    // post-order numbering
    std::vector<int> post;
    std::vector<std::pair<int, int>> stack;
    stack.push_back({broot, 0});
    while (!stack.empty()) {
        auto& top = stack.back();
        if (top.second < (int)bchildren[top.first].size()) {
            int c = bchildren[top.first][top.second++];
            stack.push_back({c, 0});
        } else {
            post.push_back(top.first);
            stack.pop_back();
        }
    }
    std::vector<int> newid(nb);
    for (int i = 0; i < nb; i++) newid[post[i]] = i;
    int s = 0;
    mb.blocks.resize(nb);
    for (int i = 0; i < nb; i++) {
        int b = post[i];
        nm_block& B = mb.blocks[i];
        B.seg = tb[b].seg;
        B.length = (int)tb[b].segs.size();
        B.s0 = s; s += B.length;
        B.parent = bparent[b] >= 0 ? newid[bparent[b]] : -1;
        B.mult = 1;
        B.degeneracy = 1.0;
        B.n_child = (int)bchildren[b].size();
        B.child0 = (int)mb.child_index.size();
        for (int c : bchildren[b]) mb.child_index.push_back(newid[c]);
        B.molmon = -1;
    }
    mb.n_store = s;
    (void)H;
    return true;
}

// Dendrimer `@dend(bp,(arm),f; ...)`: generations separated by ';'; in each,
// a branch-point segment followed by one or more pairs `(arm runs),f`, f
// copies of that arm (molecule.cpp:1437-1560; mol_dendrimer.cpp:113-184 for
// one arm type per generation, mol_asym_dendrimer.cpp:128-240 for several).
// Every arm, whatever its type, ends at a branch point of the next
// generation.  The backward propagator that reaches a next-generation branch
// point depends on the arm it came through, so the block tree holds one copy
// of the next generation under each arm type (the reference recurses into
// the next generation once per arm type, mol_asym_dendrimer.cpp:221): the
// arm type's first run carries mult = f (the join raises its end
// propagator to the f-th power), and every block of a copy the degeneracy
// of that copy, so the copies' degeneracies add up to the reference's d_mon.
// `written`: segment types in written order (generation by generation, the
// branch point, then the arms' runs), for the molecule's monomer list.
static bool build_dendrimer(const std::string& body, const std::map<std::string, int>& segidx, MolBuild& mb,
                            std::vector<int>& written, std::string& err) {
    struct Arm { std::vector<std::pair<int, int>> runs; int f = 1; };
    struct Gen { int bp = -1; std::vector<Arm> arms; };
    std::vector<Gen> G;
    for (auto& g : split(body, ';')) {
        std::vector<std::string> a = split(trim(g), ',');
        if (a.size() < 3 || (a.size() - 1) % 2 != 0) {
            err = "dendrimer generation '" + trim(g) + "': a branch point, then pairs (arm),count";
            return false;
        }
        Gen gg;
        auto it = segidx.find(trim(a[0]));
        if (it == segidx.end()) { err = "dendrimer branch point '" + a[0] + "' is not a mon"; return false; }
        gg.bp = it->second;
        written.push_back(gg.bp);
        for (size_t k = 1; k + 1 < a.size(); k += 2) {
            Arm arm;
            CompParser cp(trim(a[k]), segidx);
            std::vector<CompParser::Item> items;
            if (!cp.parse_chain(items, false)) { err = cp.err; return false; }
            for (auto& itm : items) {
                if (itm.is_side) { err = "side chains inside dendrimer arms are not supported"; return false; }
                arm.runs.push_back({itm.seg, itm.count});
                written.push_back(itm.seg);
            }
            if (arm.runs.empty()) { err = "empty dendrimer arm"; return false; }
            if (!to_int(trim(a[k + 1]), arm.f) || arm.f < 1) {
                err = "dendrimer arm count must be a positive integer"; return false;
            }
            gg.arms.push_back(arm);
        }
        G.push_back(gg);
    }
    // the tree, root (the core's branch point) first; children in written order
    struct Node { int seg, len, mult; double d; std::vector<int> ch; };
    std::vector<Node> nodes;
    bool too_big = false;
    std::function<int(size_t, double)> grow = [&](size_t g, double d) -> int {
        const int id = (int)nodes.size();
        nodes.push_back({G[g].bp, 1, 1, d, {}});
        for (const Arm& arm : G[g].arms) {
            const double da = d * arm.f;
            int prev = id;
            for (size_t r = 0; r < arm.runs.size(); r++) {
                const int rid = (int)nodes.size();
                nodes.push_back({arm.runs[r].first, arm.runs[r].second, r == 0 ? arm.f : 1, da, {}});
                nodes[prev].ch.push_back(rid);
                prev = rid;
            }
            if (nodes.size() > 4096) { too_big = true; return id; }
            if (g + 1 < G.size()) {
                const int nb = grow(g + 1, da);
                nodes[prev].ch.push_back(nb);
            }
        }
        return id;
    };
    grow(0, 1.0);
    if (too_big) { err = "dendrimer expands to more than 4096 blocks"; return false; }
    // post-order: children before their parent, the root last
    std::vector<int> post, newid(nodes.size());
    std::vector<std::pair<int, size_t>> stack{{0, 0}};
    while (!stack.empty()) {
        auto& top = stack.back();
        if (top.second < nodes[top.first].ch.size()) {
            const int c = nodes[top.first].ch[top.second++];
            stack.push_back({c, 0});
        } else {
            post.push_back(top.first);
            stack.pop_back();
        }
    }
    for (size_t i = 0; i < post.size(); i++) newid[post[i]] = (int)i;
    std::vector<int> parent(nodes.size(), -1);
    for (size_t n = 0; n < nodes.size(); n++)
        for (int c : nodes[n].ch) parent[c] = (int)n;
    const int nb = (int)post.size();
    mb.blocks.resize(nb);
    int s = 0;
    for (int i = 0; i < nb; i++) {
        const Node& t = nodes[post[i]];
        nm_block& B = mb.blocks[i];
        B.seg = t.seg; B.length = t.len; B.s0 = s; s += t.len;
        B.parent = parent[post[i]] < 0 ? -1 : newid[parent[post[i]]];
        B.mult = t.mult;
        B.degeneracy = t.d;
        B.n_child = (int)t.ch.size();
        B.child0 = (int)mb.child_index.size();
        for (int c : t.ch) mb.child_index.push_back(newid[c]);
        B.molmon = -1;
    }
    mb.n_store = s;
    return true;
}

static bool parse_range_coord(const std::string& tok, int axis, int nl, bool frozen,
                              const int bc_low, const int bc_high, int& v, std::string& err) {
    std::string t = trim(tok);
    if (t == "firstlayer") { v = 1; return true; }
    if (t == "lastlayer") { v = nl; return true; }
    if (t == "lowerbound") {
        if (!frozen || bc_low != NM_BC_SURFACE) { err = "'lowerbound' in a range needs a frozen segment and a 'surface' boundary"; return false; }
        v = 0; return true;
    }
    if (t == "upperbound") {
        if (!frozen || bc_high != NM_BC_SURFACE) { err = "'upperbound' in a range needs a frozen segment and a 'surface' boundary"; return false; }
        v = nl + 1; return true;
    }
    if (!to_int(t, v)) { err = "range coordinate '" + t + "' not understood"; return false; }
    if (v < 0 || v > nl + 1) { err = "range coordinate out of bounds"; return false; }
    (void)axis;
    return true;
}

// pinned_range / frozen_range -> MASK (segment.cpp:248-500, LGrad*::CreateMASK)
static bool make_range_mask(const PlanHolder& H, const std::string& range_in, bool frozen,
                            std::vector<double>& mask, std::string& err) {
    const nm_plan& P = H.plan;
    int g = P.gradients;
    int nl[3] = {P.MX, P.MY, P.MZ};
    std::string range = trim(range_in);
    // single keyword forms
    auto kw = [&](const std::string& k) -> std::string {
        std::string axes[3] = {"_x", "_y", "_z"};
        for (int a = 0; a < 3; a++) {
            if (k == "firstlayer" + axes[a] || k == "lastlayer" + axes[a] ||
                k == "lowerbound" + axes[a] || k == "upperbound" + axes[a]) {
                std::string base = k.substr(0, k.size() - 2);
                std::vector<std::string> lo(g), hi(g);
                for (int b = 0; b < g; b++) {
                    if (b == a) { lo[b] = base; hi[b] = base; }
                    else { lo[b] = "1"; hi[b] = std::to_string(nl[b]); }
                }
                std::string r;
                for (int b = 0; b < g; b++) r += (b ? "," : "") + lo[b];
                r += ";";
                for (int b = 0; b < g; b++) r += (b ? "," : "") + hi[b];
                return r;
            }
        }
        return "";
    };
    if (range.find(';') == std::string::npos) {
        std::string r = kw(range);
        if (r.empty()) r = kw(range + "_x");
        if (r.empty()) { err = "range '" + range + "' not understood"; return false; }
        range = r;
    }
    std::vector<std::string> ends = split(range, ';');
    if (ends.size() != 2) { err = "range must be 'lo;hi'"; return false; }
    std::vector<std::string> lo = split(ends[0], ','), hi = split(ends[1], ',');
    if ((int)lo.size() != g || (int)hi.size() != g) {
        // reference expands a single keyword coordinate of the first axis
        if ((int)lo.size() == 1 && (int)hi.size() == 1 && g > 1) {
            std::string r = kw(trim(lo[0]) + "_x");
            if (r.empty()) { err = "range needs one coordinate per gradient"; return false; }
            ends = split(r, ';'); lo = split(ends[0], ','); hi = split(ends[1], ',');
        } else { err = "range needs one coordinate per gradient"; return false; }
    }
    int a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
    for (int d = 0; d < g; d++) {
        if (!parse_range_coord(lo[d], d, nl[d], frozen, P.bc[d], P.bc[d + 3], a[d], err)) return false;
        if (!parse_range_coord(hi[d], d, nl[d], frozen, P.bc[d], P.bc[d + 3], b[d], err)) return false;
        if (a[d] > b[d]) { err = "range lower corner above upper corner"; return false; }
    }
    mask.assign(P.M, 0.0);
    for (int x = a[0]; x <= b[0]; x++)
        for (int y = (g > 1 ? a[1] : 0); y <= (g > 1 ? b[1] : 0); y++)
            for (int z = (g > 2 ? a[2] : 0); z <= (g > 2 ? b[2] : 0); z++)
                mask[x * P.JX + y * P.JY + z] = 1.0;
    return true;
}

static bool setup_lattice(const InputBlock& in, PlanHolder& H, std::string& err) {
    nm_plan& P = H.plan;
    auto lats = in.order("lat");
    if (lats.size() != 1) { err = "exactly one 'lat' is required"; return false; }
    std::string ln = lats[0];
    auto get = [&](const char* k, const char* d = "") { return in.get("lat", ln, k, d); };
    int g = 1;
    if (!to_int(get("gradients", "1"), g) || g < 1 || g > 3) { err = "lat gradients must be 1..3"; return false; }
    P.gradients = g;
    std::string lt = get("lattice_type");
    if (lt == "simple_cubic") { P.lattice_type = NM_SIMPLE_CUBIC; P.lambda = 1.0 / 6.0; }
    else if (lt == "hexagonal") { P.lattice_type = NM_HEXAGONAL; P.lambda = 1.0 / 4.0; }
    else { err = "lat lattice_type must be simple_cubic or hexagonal"; return false; }
    std::string geo = get("geometry", "planar");
    if (geo == "flat" || geo == "planar") P.geometry = NM_PLANAR;
    else if (geo == "cylindrical") P.geometry = NM_CYLINDRICAL;
    else if (geo == "spherical") P.geometry = NM_SPHERICAL;
    else { err = "lat geometry not understood"; return false; }
    if (in.has("lat", ln, "FJC_choices") || in.has("lat", ln, "b/l")) {
        std::string v = in.has("lat", ln, "b/l") ? get("b/l") : get("FJC_choices");
        if (v != "1" && v != "3") { err = "FJC_choices > 3 (fjc > 1) is not supported"; return false; }
    }
    if (in.has("lat", ln, "Markov") && get("Markov") != "1") { err = "Markov 2 chains are not supported"; return false; }
    P.stencil_full = 1;
    if (in.has("lat", ln, "stencil_full")) {
        std::string v = get("stencil_full");
        P.stencil_full = (v == "true" || v == "TRUE" || v == "1") ? 1 : 0;
    }
    if (!P.stencil_full) { err = "stencil_full : false is not supported"; return false; }
    P.offset_first_layer = 0;
    if (P.geometry != NM_PLANAR) {
        double o = 0; to_real(get("offset_first_layer", "0"), o);
        if (o < 0) o = 0;
        P.offset_first_layer = o;
    }
    P.bond_length = 0;
    if (in.has("lat", ln, "bondlength")) to_real(get("bondlength"), P.bond_length);
    bool ok = true;
    P.MX = P.MY = P.MZ = 0;
    for (int i = 0; i < 6; i++) P.bc[i] = NM_BC_MIRROR;
    if (g == 1) {
        if (!to_int(get("n_layers"), P.MX) || P.MX < 1) { err = "lat n_layers required"; return false; }
        if (in.has("lat", ln, "lowerbound")) P.bc[0] = bc_code(get("lowerbound"), ok);
        if (in.has("lat", ln, "upperbound")) P.bc[3] = bc_code(get("upperbound"), ok);
        P.JX = 1; P.JY = 0; P.M = P.MX + 2;
    } else {
        if (!to_int(get("n_layers_x"), P.MX) || P.MX < 1) { err = "lat n_layers_x required"; return false; }
        if (!to_int(get("n_layers_y"), P.MY) || P.MY < 1) { err = "lat n_layers_y required"; return false; }
        const char* lk[3] = {"lowerbound_x", "lowerbound_y", "lowerbound_z"};
        const char* uk[3] = {"upperbound_x", "upperbound_y", "upperbound_z"};
        for (int d = 0; d < g; d++) {
            if (in.has("lat", ln, lk[d])) P.bc[d] = bc_code(get(lk[d]), ok);
            if (in.has("lat", ln, uk[d])) P.bc[d + 3] = bc_code(get(uk[d]), ok);
        }
        if (g == 2) {
            if (P.geometry == NM_SPHERICAL) { err = "spherical geometry needs 1 gradient"; return false; }
            P.JX = P.MY + 2; P.JY = 1; P.M = (P.MX + 2) * (P.MY + 2);
        } else {
            if (!to_int(get("n_layers_z"), P.MZ) || P.MZ < 1) { err = "lat n_layers_z required"; return false; }
            if (P.geometry != NM_PLANAR) { err = "3 gradients need planar geometry"; return false; }
            // the reference's input check (lattice.cpp:513-516): a 3-D wall
            // is a frozen layer inside the system, not a 'surface' bound
            for (int d = 0; d < 6; d++)
                if (P.bc[d] == NM_BC_SURFACE) { err = "3-gradient lattices take mirror or periodic bounds"; return false; }
            P.JX = (P.MY + 2) * (P.MZ + 2); P.JY = P.MZ + 2; P.M = (P.MX + 2) * (P.MY + 2) * (P.MZ + 2);
        }
    }
    if (!ok) { err = "boundary condition not understood (mirror, periodic, surface)"; return false; }
    for (int d = 0; d < 3; d++)
        if ((P.bc[d] == NM_BC_PERIODIC) != (P.bc[d + 3] == NM_BC_PERIODIC)) {
            err = "a periodic boundary must be set on both sides"; return false;
        }
    // curvature weights (LGrad1.cpp:16-70 for 1 gradient, LGrad2.cpp:13-50 for 2)
    int M = P.M;
    H.L.assign(M, 0.0);
    if (P.geometry == NM_PLANAR) {
        if (g == 1) for (int i = 1; i <= P.MX; i++) H.L[i] = 1.0;   // LG1Planar.cpp:11-12
        else for (int i = 0; i < M; i++) H.L[i] = 1.0;              // LG2Planar.cpp:16-19 (3-D: unused)
        P.lambda_1 = P.lambda0 = P.lambda1 = nullptr;
    } else {
        H.lm1.assign(M, 0.0); H.l0.assign(M, 0.0); H.lp1.assign(M, 0.0);
        double lam = P.lambda;
        int ny = (g == 2) ? P.MY : 1;
        for (int x = 1; x <= P.MX; x++)
            for (int yy = 1; yy <= ny; yy++) {
                int i = (g == 2) ? x * P.JX + yy : x;
                double r = P.offset_first_layer + 1.0 * x;
                if (P.geometry == NM_CYLINDRICAL) {
                    H.L[i] = PIE * (std::pow(r, 2) - std::pow(r - 1, 2));
                    H.lp1[i] = 2.0 * PIE * r / H.L[i] * lam;
                    H.lm1[i] = 2.0 * PIE * (r - 1) / H.L[i] * lam;
                    H.l0[i] = 1.0 - 2.0 * lam;
                } else {
                    H.L[i] = 4.0 / 3.0 * PIE * (std::pow(r, 3) - std::pow(r - 1, 3));
                    H.lp1[i] = 4.0 * PIE * std::pow(r, 2) / H.L[i] * lam;
                    H.lm1[i] = 4.0 * PIE * std::pow(r - 1, 2) / H.L[i] * lam;
                    H.l0[i] = 1.0 - H.lp1[i] - H.lm1[i];
                }
            }
        P.lambda_1 = H.lm1.data(); P.lambda0 = H.l0.data(); P.lambda1 = H.lp1.data();
    }
    P.L = H.L.data();
    // volume (LGrad1.cpp PutM, LGrad2.cpp PutM, LGrad3.cpp PutM)
    if (g == 1) {
        if (P.geometry == NM_PLANAR) P.volume = P.MX;
        else if (P.geometry == NM_SPHERICAL)
            P.volume = 4.0 / 3.0 * PIE * (std::pow(P.MX + P.offset_first_layer, 3) - std::pow(P.offset_first_layer, 3));
        else P.volume = PIE * (std::pow(P.MX + P.offset_first_layer, 2) - std::pow(P.offset_first_layer, 2));
    } else if (g == 2) {
        if (P.geometry == NM_CYLINDRICAL)
            P.volume = P.MY * PIE * (std::pow(P.MX + P.offset_first_layer, 2) - std::pow(P.offset_first_layer, 2));
        else P.volume = (double)P.MX * P.MY;
    } else P.volume = (double)P.MX * P.MY * P.MZ;
    return true;
}

// Keys the compiler did not read.  The reference refuses a key outside each
// class's list (Input::CheckParameters, input.cpp:366-431).  Here a key of
// the reference's lists is accepted unread only where it cannot change a DIIS
// solve of this path: verbosity, the storage schedule, output requests, the
// guess files (the caller passes the field), the parameters of the other
// Newton methods (sfnewton.cpp; iterate_DIIS reads none of them) and of the
// outer loop of constraints (refused themselves).  Any other key is refused
// by name, so an input that relies on a feature this library does not have
// cannot run with it silently dropped.
static bool no_effect(const Entry& e) {
    static const char* const newton_keys[] = {
        "x_info", "e_info", "s_info", "i_info", "t_info", "hs_info", "super_e_info", "super_s_info",
        "super_i_info", "super_tolerance", "super_iterationlimit", "super_deltamax", "deltamin",
        "linesearchlimit", "samehessian", "max_accuracy_for_hessian_scaling", "n_iterations_for_hessian",
        "small_alpha", "target_function", "max_n_small_alpha", "min_accuracy_for_hessian",
        "max_fr_reverse_direction", "print_hessian_at_it"};
    static const char* const sys_keys[] = {"GPU", "initial_guess", "guess_inputfile", "final_guess",
                                           "guess_outputfile"};
    if (e.cls == "output") return true;
    if (e.cls == "mol") return e.key == "save_memory";
    if (e.cls == "newton") {
        if (e.key == "gradient_type") return e.value == "classical";
        for (const char* k : newton_keys) if (e.key == k) return true;
        return false;
    }
    if (e.cls == "sys") {
        if (e.key == "calculation_type") return e.value == "equilibrium";
        for (const char* k : sys_keys) if (e.key == k) return true;
        return false;
    }
    return false;
}

static bool check_unread(const InputBlock& in, std::string& err) {
    for (auto& e : in.entries) {
        if (e.used || no_effect(e)) continue;
        err = "input key not supported here (it would change the solve or needs a feature outside this path): '" +
              e.cls + " : " + e.name + " : " + e.key + "'";
        return false;
    }
    return true;
}

// ---- internal states and reactions ----------------------------------------

// The states' bulk fractions as the reference fixes them before its SCF
// loop (Solve_scf::Solve, solve_scf.cpp:562-603): one unknown x_r per
// reaction, the residual of the WEAK case of Solve_scf::residuals
// (solve_scf.cpp:762-785) — every reaction's analytic guess (3-term
// reactions first), then each reaction scales its segment's iterated state
// by exp(x_r), then g_r = -1 + Σ -ν·log10(α_bulk)/pK_eff.
struct Chem {
    const std::vector<ReactionDef>& R;
    std::vector<double> pke;           // pK_eff of each reaction
    const std::vector<int>& seg;       // segment of each state
    const std::vector<double>& val;    // valence of each state
    const std::vector<char>& fixed;    // alphabulk given in the input
    std::vector<std::vector<int>> seg_states;
    std::vector<int> local;            // index of a state within its segment
    std::vector<double> ab;            // α_bulk of each state
    std::vector<int> item;             // Segment::ItState of each segment
    std::string err;

    Chem(const std::vector<ReactionDef>& r, const std::vector<int>& s, const std::vector<double>& v,
         const std::vector<char>& f, const std::vector<double>& ab0, int n_seg)
        : R(r), pke(r.size()), seg(s), val(v), fixed(f), seg_states(n_seg), local(s.size()), ab(ab0), item(n_seg, -1) {
        for (size_t i = 0; i < r.size(); i++) pke[i] = r[i].pK;
        for (size_t j = 0; j < s.size(); j++) {
            local[j] = (int)seg_states[s[j]].size();
            seg_states[s[j]].push_back((int)j);
        }
    }
    // pK_eff = pK + Σ ν·ChemIntBulk/ln 10 (reaction.cpp:253-266): pke, set
    // by the caller (pK itself before any solve, when the bulk fractions the
    // χ sums read are still zero)
    double pK_eff(const ReactionDef& r) const { return pke[&r - R.data()]; }

    // Reaction::GuessAlpha, reaction.cpp:300-378
    bool guess(const ReactionDef& r) {
        const int n = (int)r.sto.size();
        double k = std::pow(10.0, -pK_eff(r));
        if (n == 3) {
            int water = -1;
            double af = -1;
            for (int i = 0; i < n; i++)
                if (fixed[r.state[i]]) { water = seg[r.state[i]]; af = ab[r.state[i]]; }
            if (water < 0 || seg_states[water].size() != 3) {
                err = "reaction " + r.name + ": a 3-term reaction needs one segment with three states, one of "
                      "them with a fixed alphabulk";
                return false;
            }
            double sum = 0;
            for (int li = 0; li < 3; li++) {
                const int s = seg_states[water][li];
                if (!fixed[s]) {
                    if (val[s] == 0) ab[s] = 0;
                    else { ab[s] = k / af; item[water] = li; }
                }
                sum += ab[s];
            }
            for (int li = 0; li < 3; li++) {
                const int s = seg_states[water][li];
                if (!fixed[s] && val[s] == 0) ab[s] = 1 - sum;
            }
            return true;
        }
        int water = -1, other = -1;
        for (int i = 0; i < n; i++) if (fixed[r.state[i]]) water = seg[r.state[i]];
        for (int i = 0; i < n; i++) if (seg[r.state[i]] != water) other = seg[r.state[i]];
        if (water < 0 || other < 0) {
            err = "reaction " + r.name + ": needs the states of one segment with a fixed alphabulk and of one other";
            return false;
        }
        int s1 = -1, s2 = -1;
        for (int i = 0; i < n; i++) {
            const int s = r.state[i];
            if (seg[s] == water) { k = k / std::pow(ab[s], r.sto[i]); continue; }
            if (seg[s] != other) {
                err = "reaction " + r.name + ": states of more than two segments";
                return false;
            }
            if (s1 < 0) { s1 = local[s]; continue; }
            if (s2 >= 0 || r.sto[i] <= 0) {
                err = "reaction " + r.name + ": needs exactly two states of its other segment, the second "
                      "on the right-hand side";
                return false;
            }
            s2 = local[s];
            item[other] = s2;
        }
        if (s2 < 0) { err = "reaction " + r.name + ": needs two states of its other segment"; return false; }
        ab[seg_states[other][s2]] = k / (k + 1);
        ab[seg_states[other][s1]] = 1 / (k + 1);
        return true;
    }
    // Reaction::PutAlpha (reaction.cpp:285-298) and Segment::PutAlpha
    // (segment.cpp:2052-2080)
    bool put_alpha(const ReactionDef& r, double a) {
        const int n = (int)r.sto.size();
        int water = -1, other = -1;
        for (int i = 0; i < n; i++) if (fixed[r.state[i]]) water = seg[r.state[i]];
        for (int i = 0; i < n; i++) if (seg[r.state[i]] != water) other = seg[r.state[i]];
        const int sg = other > -1 ? other : water;
        const std::vector<int>& st = seg_states[sg];
        const int it = item[sg];
        if (st.size() < 2 || it < 0) {
            err = "reaction " + r.name + ": no iterated state for its segment";
            return false;
        }
        for (int li = 0; li < (int)st.size(); li++)
            if (li != it && !fixed[st[li]]) ab[st[li]] = 0;
        ab[st[it]] *= a;
        double sum = 0;
        for (int s : st) sum += ab[s];
        bool ok = true;
        for (int s : st) {
            if (ab[s] == 0) ab[s] = 1.0 - sum;
            if (ab[s] < 0 || ab[s] > 1) ok = false;
        }
        if (!ok) err = "reaction " + r.name + ": a bulk fraction (alphabulk) left [0, 1]";
        return ok;
    }
    // Reaction::Residual_value, reaction.cpp:269-284
    double residual(const ReactionDef& r) const {
        double res = 0;
        for (size_t i = 0; i < r.sto.size(); i++) {
            const double a = ab[r.state[i]];
            if (a > 0) res -= r.sto[i] * std::log10(a);
        }
        return -1.0 + res / pK_eff(r);
    }
    bool weak(const std::vector<double>& x, std::vector<double>& g) {
        for (auto& r : R) if (r.sto.size() == 3 && !guess(r)) return false;
        for (auto& r : R) if (r.sto.size() != 3 && !guess(r)) return false;
        for (size_t i = 0; i < R.size(); i++) if (!put_alpha(R[i], std::exp(x[i]))) return false;
        for (size_t i = 0; i < R.size(); i++) g[i] = residual(R[i]);
        return true;
    }
    static double norm(const std::vector<double>& g) {
        double s = 0;
        for (double v : g) s += v * v;
        return std::sqrt(s);
    }
    // The reference's Newton (SFNewton::iterate with tolerance 1e-8, at most
    // 100 steps) takes no step when the residual at the guesses is small;
    // the guesses are then the result.  Runs of the reference on the
    // autoprotolysis/weak-acid pair at pK_w 14 and 16 and H3O+ fractions
    // from 1e-9 to 1e-3 put that bound at |g| between 1.35e-8 (no step) and
    // 1.41e-8 (steps).  When it steps it ends at the root to rounding (its
    // bulk fractions agree with the root to 1e-12), and this Newton with a
    // central-difference Jacobian and step halving goes to the same root.
    bool solve() {
        const int n = (int)R.size();
        std::vector<double> x(n, 0.0), g(n), gp(n), gm(n), xn(n), gn(n);
        if (!weak(x, g)) return false;
        if (norm(g) <= 1.38e-8) return true;
        for (int it = 0; it < 100 && norm(g) > 1e-15; it++) {
            std::vector<double> J((size_t)n * n), p(n);
            const double h = 1e-6;
            for (int j = 0; j < n; j++) {
                std::vector<double> xp = x, xm = x;
                xp[j] += h; xm[j] -= h;
                if (!weak(xp, gp) || !weak(xm, gm)) return false;
                for (int i = 0; i < n; i++) J[(size_t)i * n + j] = (gp[i] - gm[i]) / (2 * h);
            }
            for (int i = 0; i < n; i++) p[i] = -g[i];
            for (int c = 0; c < n; c++) {  // elimination with partial pivoting
                int pr = c;
                for (int r = c + 1; r < n; r++) if (std::fabs(J[(size_t)r * n + c]) > std::fabs(J[(size_t)pr * n + c])) pr = r;
                if (J[(size_t)pr * n + c] == 0) { err = "bulk equilibrium of the reactions: singular Jacobian"; return false; }
                if (pr != c) {
                    for (int k = 0; k < n; k++) std::swap(J[(size_t)pr * n + k], J[(size_t)c * n + k]);
                    std::swap(p[pr], p[c]);
                }
                for (int r = c + 1; r < n; r++) {
                    const double f = J[(size_t)r * n + c] / J[(size_t)c * n + c];
                    for (int k = c; k < n; k++) J[(size_t)r * n + k] -= f * J[(size_t)c * n + k];
                    p[r] -= f * p[c];
                }
            }
            for (int c = n - 1; c >= 0; c--) {
                for (int k = c + 1; k < n; k++) p[c] -= J[(size_t)c * n + k] * p[k];
                p[c] /= J[(size_t)c * n + c];
            }
            double t = 1;
            bool better = false;
            for (int ls = 0; ls < 30; ls++, t *= 0.5) {
                for (int i = 0; i < n; i++) xn[i] = x[i] + t * p[i];
                if (weak(xn, gn) && norm(gn) < norm(g)) { better = true; break; }
            }
            if (!better) break;
            x = xn; g = gn;
        }
        if (!weak(x, g)) return false;
        if (norm(g) > 1e-8) { err = "bulk equilibrium of the reactions did not converge"; return false; }
        return true;
    }
};

// States, reactions, the species χ matrix and the states' bulk fractions.
// Runs after the segments' χ are resolved and before the molecules.
static bool build_states(const InputBlock& in, PlanHolder& H, std::string& err) {
    nm_plan& P = H.plan;
    const int ns = P.n_seg;
    H.state_names = in.order("state");
    const int nst = (int)H.state_names.size();
    H.seg_nstate.assign(ns, 0);
    if (nst == 0) {
        if (!in.order("reaction").empty()) { err = "reactions need internal states ('state' keys)"; return false; }
        return true;
    }
    // System::CheckInput marks internal states only for two or more
    // (system.cpp:1044); one state alone has no species of its own
    if (nst == 1) { err = "a single internal state is not supported (define two or more)"; return false; }
    std::map<std::string, int> segidx, stidx;
    for (int i = 0; i < ns; i++) segidx[H.seg_names[i]] = i;
    for (int j = 0; j < nst; j++) {
        if (segidx.count(H.state_names[j])) {
            err = "state " + H.state_names[j] + ": a state's name cannot be a mon's name"; return false;
        }
        stidx[H.state_names[j]] = j;
    }
    // State::CheckInput, state.cpp:37-106
    H.state_seg.assign(nst, -1);
    H.state_valence.assign(nst, 0.0);
    std::vector<double> ab0(nst, -1.0);
    std::vector<char> fixed(nst, 0);
    for (int j = 0; j < nst; j++) {
        const std::string& sn = H.state_names[j];
        const std::string mon = in.get("state", sn, "mon");
        if (mon.empty()) { err = "state " + sn + " needs its 'mon'"; return false; }
        if (!segidx.count(mon)) { err = "state " + sn + ": mon " + mon + " not found"; return false; }
        const int sg = segidx[mon];
        if (H.seg_freedom[sg] == NM_SEG_FROZEN) { err = "state " + sn + ": states of a frozen mon are not supported"; return false; }
        H.state_seg[j] = sg;
        H.seg_nstate[sg]++;
        if (in.has("state", sn, "alphabulk")) {
            if (!to_real(in.get("state", sn, "alphabulk"), ab0[j]) || ab0[j] < 0 || ab0[j] > 1) {
                err = "state " + sn + ": alphabulk out of range 0 ... 1"; return false;
            }
            fixed[j] = 1;
        }
        if (in.has("state", sn, "valence")) {
            double v = 0;
            if (!to_real(in.get("state", sn, "valence"), v) || v < -10 || v > 10) {
                err = "state " + sn + ": valence out of range -10 ... 10"; return false;
            }
            H.state_valence[j] = v;
        }
    }
    for (int i = 0; i < ns; i++)
        if (H.seg_nstate[i] == 1) {
            err = "mon " + H.seg_names[i] + " has a single internal state (define two or more, or none)"; return false;
        }
    // reactions (Reaction::CheckInput, reaction.cpp:37-145)
    std::vector<ReactionDef> R;
    for (const std::string& rn : in.order("reaction")) {
        ReactionDef r;
        r.name = rn;
        const bool hK = in.has("reaction", rn, "K"), hpK = in.has("reaction", rn, "pK");
        if (!hK && !hpK) { err = "reaction " + rn + " has no K nor pK value"; return false; }
        if (!hK) {
            if (!to_real(in.get("reaction", rn, "pK"), r.pK)) { err = "reaction " + rn + ": no valid pK value"; return false; }
        } else {
            double K = -1;
            if (!to_real(in.get("reaction", rn, "K"), K) || K < 0) { err = "reaction " + rn + ": K must be positive"; return false; }
            r.pK = -std::log10(K);
        }
        const std::string eq = in.get("reaction", rn, "equation");
        if (eq.empty()) { err = "reaction " + rn + " has no equation"; return false; }
        std::vector<std::string> sides = split(eq, '=');
        if (sides.size() != 2) { err = "reaction " + rn + ": the equation needs one '=' sign"; return false; }
        for (int side = 0; side < 2; side++)
            for (const std::string& t0 : split(sides[side], '+')) {
                const std::string t = trim(t0);
                const size_t o = t.find('('), c = t.rfind(')');
                if (o == std::string::npos || c == std::string::npos || c < o || t.find('(', o + 1) != std::string::npos) {
                    err = "reaction " + rn + ": term '" + t + "' is not of the form n(state)"; return false;
                }
                const std::string name = trim(t.substr(o + 1, c - o - 1));
                if (!stidx.count(name)) { err = "reaction " + rn + ": state " + name + " not found"; return false; }
                int sto = 0;
                if (!to_int(trim(t.substr(0, o)), sto) || sto < 1) {
                    err = "reaction " + rn + ": stoichiometric numbers are positive integers"; return false;
                }
                r.state.push_back(stidx[name]);
                r.sto.push_back(side == 0 ? -sto : sto);
            }
        for (int i = 0; i < ns; i++) {  // balanced per mon
            int sum = 0;
            for (size_t k = 0; k < r.sto.size(); k++) if (H.state_seg[r.state[k]] == i) sum += r.sto[k];
            if (sum != 0) { err = "reaction " + rn + ": not balanced for the states of mon " + H.seg_names[i]; return false; }
        }
        double q = 0;
        for (size_t k = 0; k < r.sto.size(); k++) q += r.sto[k] * H.state_valence[r.state[k]];
        if (std::fabs(q) > 1e-10) { err = "reaction " + rn + ": not electroneutral"; return false; }
        R.push_back(r);
    }
    // system.cpp:1044-1083: one equation or fixed alphabulk per state beyond
    // the first of each segment
    int n_fixed = 0, n_segs = 0;
    for (int j = 0; j < nst; j++) n_fixed += fixed[j];
    for (int i = 0; i < ns; i++) n_segs += H.seg_nstate[i] > 1;
    if (n_segs + (int)R.size() + n_fixed != nst) {
        err = "internal states: (mons with states) + (reactions) + (fixed alphabulk values) must equal the number "
              "of states";
        return false;
    }
    Chem chem(R, H.state_seg, H.state_valence, fixed, ab0, ns);
    if (!chem.solve()) { err = chem.err; return false; }
    H.reactions = R;
    H.state_fixed = fixed;
    H.state_ab_in = ab0;
    for (int j = 0; j < nst; j++)
        if (!(chem.ab[j] >= 0 && chem.ab[j] <= 1)) {
            err = "state " + H.state_names[j] + ": its bulk fraction is fixed by no reaction"; return false;
        }
    H.state_alphabulk = chem.ab;
    // χ between species (system.cpp:1775-1915): the segments' resolved
    // matrix, then state–state and segment–state pairs; an unset pair takes
    // the value of the states' mons, a pair set once is symmetric
    const int nsp = ns + nst;
    const double UNSET = -999;
    H.chi_sp.assign((size_t)nsp * nsp, UNSET);
    for (int i = 0; i < ns; i++)
        for (int k = 0; k < ns; k++) H.chi_sp[(size_t)i * nsp + k] = H.chi[(size_t)i * ns + k];
    auto name_of = [&](int a) { return a < ns ? H.seg_names[a] : H.state_names[a - ns]; };
    for (int a = 0; a < nsp; a++)
        for (int b = ns; b < nsp; b++) {
            if (a < ns && b < ns) continue;
            const std::string key = "chi_" + name_of(b);
            const char* cls = a < ns ? "mon" : "state";
            if (!in.has(cls, name_of(a), key)) continue;
            double v;
            if (!to_real(in.get(cls, name_of(a), key), v)) { err = "chi value not a number"; return false; }
            if (a == b) v = 0;  // state.cpp:102: χ of a state with itself is ignored
            H.chi_sp[(size_t)a * nsp + b] = v;
        }
    for (int a = ns; a < nsp; a++)  // state rows toward segments
        for (int k = 0; k < ns; k++) {
            const std::string key = "chi_" + H.seg_names[k];
            if (!in.has("state", H.state_names[a - ns], key)) continue;
            double v;
            if (!to_real(in.get("state", H.state_names[a - ns], key), v)) { err = "chi value not a number"; return false; }
            H.chi_sp[(size_t)a * nsp + k] = v;
        }
    auto mon_of = [&](int a) { return a < ns ? a : H.state_seg[a - ns]; };
    for (int a = 0; a < nsp; a++)
        for (int b = 0; b < nsp; b++) {
            if (a < ns && b < ns) continue;
            double& ab_ = H.chi_sp[(size_t)a * nsp + b];
            double& ba = H.chi_sp[(size_t)b * nsp + a];
            if (ab_ == UNSET && ba == UNSET) ab_ = ba = H.chi[(size_t)mon_of(a) * ns + mon_of(b)];
            else if (ab_ != UNSET && ba == UNSET) ba = ab_;
            else if (ab_ == UNSET && ba != UNSET) ab_ = ba;
            else if (ab_ != ba) { err = "conflict in chi values between " + name_of(a) + " and " + name_of(b); return false; }
        }
    for (int j = 0; j < nst; j++) {
        const int sg = H.state_seg[j];
        if (H.chi_sp[(size_t)sg * nsp + ns + j] != 0) {
            err = "chi between a mon and one of its own states (" + H.state_names[j] + ") is not allowed"; return false;
        }
    }
    // the states carry the charge of a mon with states (System::
    // DoElectrostatics, system.cpp:1921-1941; PutU, :1985-2080)
    for (int i = 0; i < ns; i++) if (H.seg_nstate[i] > 0) H.seg_valence[i] = 0;
    P.n_state = nst;
    P.n_sp = nsp;
    return true;
}

std::vector<double> plan_reaction_pK(const nm_plan* p) {
    const PlanHolder& H = *reinterpret_cast<const PlanHolder*>(p);
    std::vector<double> pk;
    for (auto& r : H.reactions) pk.push_back(r.pK);
    return pk;
}

int plan_reaction_index(const nm_plan* p, const std::string& name) {
    const PlanHolder& H = *reinterpret_cast<const PlanHolder*>(p);
    for (size_t r = 0; r < H.reactions.size(); r++)
        if (H.reactions[r].name == name) return (int)r;
    return -1;
}

int plan_state_bulk(const nm_plan* p, const std::vector<double>& fixed_ab, const std::vector<double>& pK,
                    const double* sp_phibulk, std::vector<double>& alphabulk, std::vector<double>& mol_charge,
                    std::string& err) {
    const PlanHolder& H = *reinterpret_cast<const PlanHolder*>(p);
    const int ns = p->n_seg, nst = p->n_state, nsp = p->n_sp;
    if (nst == 0 || (int)fixed_ab.size() != nst || pK.size() != H.reactions.size()) {
        err = "no internal states";
        return NM_ERR_ARG;
    }
    std::vector<ReactionDef> R = H.reactions;
    for (size_t r = 0; r < R.size(); r++) R[r].pK = pK[r];
    std::vector<double> ab0 = H.state_ab_in;
    for (int j = 0; j < nst; j++)
        if (H.state_fixed[j]) {
            if (!(fixed_ab[j] >= 0 && fixed_ab[j] <= 1)) { err = "alphabulk out of range 0 ... 1"; return NM_ERR_ARG; }
            ab0[j] = fixed_ab[j];
        }
    Chem chem(R, H.state_seg, H.state_valence, H.state_fixed, ab0, ns);
    if (sp_phibulk) {
        // Reaction::pKeff (reaction.cpp:253-266) with ChemIntBulk
        // (reaction.cpp:243-251) over the bulk volume fractions of the last
        // solve; the reference indexes the states by the term's position in
        // the equation (Sta[i]), and so does this
        auto cib = [&](int j) {
            double v = 0;
            for (int k = 0; k < ns; k++)
                if (H.seg_nstate[k] == 0) v += p->chi_sp[(size_t)(ns + j) * nsp + k] * sp_phibulk[k];
            for (int l = 0; l < nst; l++) v += p->chi_sp[(size_t)(ns + j) * nsp + ns + l] * sp_phibulk[ns + l];
            return v;
        };
        for (size_t r = 0; r < R.size(); r++) {
            double v = 0;
            for (size_t i = 0; i < R[r].sto.size() && (int)i < nst; i++) v += R[r].sto[i] * cib((int)i);
            chem.pke[r] = R[r].pK + v / std::log(10.0);
        }
    }
    if (!chem.solve()) { err = chem.err; return NM_ERR_INPUT; }
    for (int j = 0; j < nst; j++)
        if (!(chem.ab[j] >= 0 && chem.ab[j] <= 1)) { err = "a state's bulk fraction left [0, 1]"; return NM_ERR_INPUT; }
    alphabulk = chem.ab;
    // Molecule::Charge with the new fractions, as the plan computes it
    mol_charge.assign(p->n_mol, 0.0);
    size_t off = 0;
    for (int m = 0; m < p->n_mol; m++) {
        const nm_molecule& mol = p->mols[m];
        bool with_states = false;
        for (int k = 0; k < mol.n_molmon; k++) with_states = with_states || H.seg_nstate[mol.molmon_seg[k]] > 0;
        if (!with_states) {
            mol_charge[m] = mol.charge;
        } else {
            double q = 0;
            for (int k = 0; k < mol.n_molmon; k++) {
                const int sgi = mol.molmon_seg[k];
                const double nmon = H.mol_nmon[off + k];
                if (H.seg_nstate[sgi] > 0) {
                    for (int j = 0; j < nst; j++)
                        if (H.state_seg[j] == sgi) q += alphabulk[j] * H.state_valence[j] * nmon;
                } else q += H.seg_valence[sgi] * nmon;
            }
            mol_charge[m] = q / mol.chainlength;
        }
        off += mol.n_molmon;
    }
    return NM_OK;
}

static nm_plan* build_plan(const InputBlock& in, std::string& err) {
    PlanHolder* H = new PlanHolder();
    nm_plan& P = H->plan;
    std::memset(&P, 0, sizeof(P));
    if (!setup_lattice(in, *H, err)) { delete H; return nullptr; }
    int M = P.M;
    // ---- segments ----
    H->seg_names = in.order("mon");
    int ns = (int)H->seg_names.size();
    if (ns < 1) { err = "at least one 'mon' is required"; delete H; return nullptr; }
    std::map<std::string, int> segidx;
    for (int i = 0; i < ns; i++) segidx[H->seg_names[i]] = i;
    P.n_seg = ns;
    H->seg_freedom.assign(ns, NM_SEG_FREE);
    H->seg_valence.assign(ns, 0.0);
    H->seg_epsilon.assign(ns, 80.0);
    H->seg_mask.assign((size_t)ns * M, 0.0);
    for (int i = 0; i < ns; i++) {
        const std::string& nm_ = H->seg_names[i];
        std::string fr = in.get("mon", nm_, "freedom", "free");
        if (fr == "free") H->seg_freedom[i] = NM_SEG_FREE;
        else if (fr == "pinned") H->seg_freedom[i] = NM_SEG_PINNED;
        else if (fr == "frozen") H->seg_freedom[i] = NM_SEG_FROZEN;
        else { err = "mon " + nm_ + " freedom '" + fr + "' is not supported (free, pinned, frozen)"; delete H; return nullptr; }
        if (H->seg_freedom[i] != NM_SEG_FREE) {
            const char* key = H->seg_freedom[i] == NM_SEG_PINNED ? "pinned_range" : "frozen_range";
            if (!in.has("mon", nm_, key)) { err = "mon " + nm_ + " needs '" + key + "'"; delete H; return nullptr; }
            std::vector<double> mask;
            if (!make_range_mask(*H, in.get("mon", nm_, key), H->seg_freedom[i] == NM_SEG_FROZEN, mask, err)) {
                err = "mon " + nm_ + ": " + err; delete H; return nullptr;
            }
            std::copy(mask.begin(), mask.end(), H->seg_mask.begin() + (size_t)i * M);
        }
        if (in.has("mon", nm_, "valence")) to_real(in.get("mon", nm_, "valence"), H->seg_valence[i]);
        if (in.has("mon", nm_, "epsilon")) to_real(in.get("mon", nm_, "epsilon"), H->seg_epsilon[i]);
        if (in.has("mon", nm_, "e.psi0/kT")) {
            // the reference's fixed-ψ0 residual resets ψ to 0 off the surface at
            // every evaluation (OverwriteC, tools_host.h:515-517, from
            // Segment::UpdateValence), so it iterates no potential; not offered
            err = "mon " + nm_ + ": fixed surface potentials (e.psi0/kT) are not supported";
            delete H; return nullptr;
        }
        if (in.has("mon", nm_, "fluctuation_potentials") || in.has("mon", nm_, "state1")) {
            err = "mon " + nm_ + ": external potentials / internal states are not supported"; delete H; return nullptr;
        }
    }
    // chi (system.cpp CheckChi_values)
    H->chi.assign((size_t)ns * ns, 123.0);
    for (int i = 0; i < ns; i++)
        for (int k = 0; k < ns; k++) {
            std::string key = "chi_" + H->seg_names[k];
            if (in.has("mon", H->seg_names[i], key)) {
                double v;
                if (!to_real(in.get("mon", H->seg_names[i], key), v)) { err = "chi value not a number"; delete H; return nullptr; }
                H->chi[i * ns + k] = v;
            }
        }
    for (int i = 0; i < ns; i++) for (int k = 0; k < ns; k++)
        if (H->chi[i * ns + k] == 123.0) H->chi[i * ns + k] = H->chi[k * ns + i];
    for (int i = 0; i < ns; i++) for (int k = 0; k < ns; k++)
        if (H->chi[i * ns + k] == 123.0) H->chi[i * ns + k] = 0.0;
    for (int i = 0; i < ns; i++) {
        if (H->chi[i * ns + i] != 0) { err = "chi of a segment with itself must be zero"; delete H; return nullptr; }
        for (int k = 0; k < ns; k++)
            if (H->chi[i * ns + k] != H->chi[k * ns + i]) { err = "chi matrix must be symmetric"; delete H; return nullptr; }
    }
    if (!build_states(in, *H, err)) { delete H; return nullptr; }
    // KSAM (system.cpp generate_mask): 0 where any frozen segment sits
    H->ksam.assign(M, 1);
    for (int i = 0; i < ns; i++)
        if (H->seg_freedom[i] == NM_SEG_FROZEN)
            for (int s = 0; s < M; s++) if (H->seg_mask[(size_t)i * M + s] != 0) H->ksam[s] = 0;
    H->seg_gmask.assign((size_t)ns * M, 0.0);
    H->seg_phi_frozen.assign((size_t)ns * M, 0.0);
    for (int i = 0; i < ns; i++)
        for (int s = 0; s < M; s++) {
            double km = H->ksam[s];
            // pinned: G1 = exp(-u)·MASK·KSAM; free and frozen: exp(-u)·KSAM
            // (segment.cpp:875-878; the frozen test there compares against
            // " frozen", so frozen segments get the KSAM factor as well)
            if (H->seg_freedom[i] == NM_SEG_PINNED) H->seg_gmask[(size_t)i * M + s] = H->seg_mask[(size_t)i * M + s] * km;
            else H->seg_gmask[(size_t)i * M + s] = km;
            if (H->seg_freedom[i] == NM_SEG_FROZEN) H->seg_phi_frozen[(size_t)i * M + s] = H->seg_mask[(size_t)i * M + s];
        }
    // surface bounds must be frozen (the halo layer is then a G = 0 wall)
    for (int d = 0; d < P.gradients; d++)
        for (int side = 0; side < 2; side++) {
            if (P.bc[d + 3 * side] != NM_BC_SURFACE) continue;
            int nl[3] = {P.MX, P.MY, P.MZ};
            int layer = side ? nl[d] + 1 : 0;
            // every non-corner site of that halo layer must carry KSAM = 0
            int g = P.gradients;
            for (int x = 1; x <= P.MX; x++)
                for (int y = (g > 1 ? 1 : 0); y <= (g > 1 ? P.MY : 0); y++)
                    for (int z = (g > 2 ? 1 : 0); z <= (g > 2 ? P.MZ : 0); z++) {
                        int c[3] = {x, y, z};
                        c[d] = layer;
                        int s = c[0] * P.JX + c[1] * P.JY + c[2];
                        if (H->ksam[s] != 0) {
                            err = "a 'surface' boundary needs a frozen segment on its halo layer "
                                  "(frozen_range : lowerbound / upperbound)";
                            delete H; return nullptr;
                        }
                    }
        }
    // ---- molecules ----
    auto molnames = in.order("mol");
    int nmol = (int)molnames.size();
    if (nmol < 1) { err = "at least one 'mol' is required"; delete H; return nullptr; }
    H->mb.resize(nmol);
    P.solvent = -1; P.neutralizer = -1;
    for (int m = 0; m < nmol; m++) {
        MolBuild& mb = H->mb[m];
        const std::string& mn = molnames[m];
        std::string comp = in.get("mol", mn, "composition");
        if (comp.empty()) { err = "mol " + mn + " needs a composition"; delete H; return nullptr; }
        if (comp.find('#') != std::string::npos) { err = "aliases in compositions are not supported"; delete H; return nullptr; }
        std::string fr = in.get("mol", mn, "freedom");
        if (fr == "free") mb.mol.freedom = NM_MOL_FREE;
        else if (fr == "restricted") mb.mol.freedom = NM_MOL_RESTRICTED;
        else if (fr == "solvent") { mb.mol.freedom = NM_MOL_SOLVENT; P.solvent = m; }
        else if (fr == "neutralizer") { mb.mol.freedom = NM_MOL_NEUTRALIZER; P.neutralizer = m; }
        else { err = "mol " + mn + " freedom '" + fr + "' is not supported"; delete H; return nullptr; }
        {   // Molecule::CheckInput, molecule.cpp:369-372 (Input::Get_bool, input.cpp:270-277)
            const std::string sm = in.get("mol", mn, "save_memory", "false");
            if (sm == "true" || sm == "True" || sm == "TRUE") P.save_memory = 1;
        }
        if (mb.mol.freedom == NM_MOL_FREE) {
            if (!in.has("mol", mn, "phibulk")) { err = "free mol " + mn + " needs phibulk"; delete H; return nullptr; }
            to_real(in.get("mol", mn, "phibulk"), mb.mol.phibulk);
        }
        // parse composition
        std::vector<std::string> order_seen;
        std::vector<int> dend_written;
        if (comp.rfind("@dend(", 0) == 0) {
            if (comp.back() != ')') { err = "dendrimer composition must end with ')'"; delete H; return nullptr; }
            if (!build_dendrimer(comp.substr(6, comp.size() - 7), segidx, mb, dend_written, err)) {
                delete H; return nullptr;
            }
            mb.is_dendrimer = true;
        } else if (comp[0] == '@') {
            err = "composition keyword not supported (only @dend)"; delete H; return nullptr;
        } else {
            CompParser cp(comp, segidx);
            std::vector<CompParser::Item> items;
            if (!cp.parse_chain(items, false) || cp.pos != comp.size()) {
                err = "mol " + mn + " composition: " + (cp.err.empty() ? "trailing text" : cp.err); delete H; return nullptr;
            }
            bool branched = comp.find('[') != std::string::npos;
            std::vector<SegNode> nodes;
            std::vector<int> written;
            if (!emit_chain(items, nodes, -1, written, err)) { delete H; return nullptr; }
            if (nodes.empty()) { err = "empty composition"; delete H; return nullptr; }
            // reference roots: linear chains at the last written segment
            // (mol_linear.cpp:113-131), branched ones at the first
            // (molecule.cpp:1740-1766 reverses the numbering)
            int root = branched ? written.front() : written.back();
            if (!build_blocks_from_tree(nodes, root, *H, mb, err)) { delete H; return nullptr; }
        }
        // molmon list in written order of first appearance
        {
            std::vector<int> segs_in_order;
            if (mb.is_dendrimer) {
                // written order: generation by generation, bp then arm runs
                segs_in_order = dend_written;
            } else {
                // recover written order from the composition text
                CompParser cp(comp, segidx);
                std::vector<CompParser::Item> items;
                cp.parse_chain(items, false);
                std::function<void(const std::vector<CompParser::Item>&)> walk =
                    [&](const std::vector<CompParser::Item>& v) {
                        for (auto& it : v) { if (it.is_side) walk(it.side); else segs_in_order.push_back(it.seg); }
                    };
                walk(items);
                // branched compositions are numbered back to front
                // (molecule.cpp:1740-1766), and MolMonList follows that
                // numbering (Molecule::MakeMonList, molecule.cpp:1785-1800)
                if (comp.find('[') != std::string::npos)
                    std::reverse(segs_in_order.begin(), segs_in_order.end());
            }
            for (int sgi : segs_in_order)
                if (std::find(mb.molmon.begin(), mb.molmon.end(), sgi) == mb.molmon.end()) mb.molmon.push_back(sgi);
        }
        double N = 0;
        for (auto& B : mb.blocks) N += B.length * B.degeneracy;
        mb.mol.chainlength = N;
        mb.fraction.assign(mb.molmon.size(), 0.0);
        for (auto& B : mb.blocks) {
            int k = (int)(std::find(mb.molmon.begin(), mb.molmon.end(), B.seg) - mb.molmon.begin());
            B.molmon = k;
            mb.fraction[k] += B.length * B.degeneracy;
            if (H->seg_freedom[B.seg] == NM_SEG_FROZEN) { err = "frozen segment used in a molecule"; delete H; return nullptr; }
            if (H->seg_freedom[B.seg] == NM_SEG_PINNED) mb.mol.pinned = 1;
        }
        for (auto& f : mb.fraction) f /= N;
        {
            std::vector<double> nm(mb.molmon.size(), 0.0);
            for (auto& B : mb.blocks) {
                const int k = (int)(std::find(mb.molmon.begin(), mb.molmon.end(), B.seg) - mb.molmon.begin());
                nm[k] += B.length * B.degeneracy;
            }
            H->mol_nmon.insert(H->mol_nmon.end(), nm.begin(), nm.end());
        }
        mb.mol.charge = 0;
        bool with_states = false;
        for (int sgi : mb.molmon) with_states = with_states || H->seg_nstate[sgi] > 0;
        if (!with_states) {
            for (size_t k = 0; k < mb.molmon.size(); k++) mb.mol.charge += mb.fraction[k] * H->seg_valence[mb.molmon[k]];
        } else {
            // Molecule::Charge (molecule.cpp:1866-1879): a mon with states
            // counts Σ α_bulk·valence of its states
            double q = 0;
            for (size_t k = 0; k < mb.molmon.size(); k++) {
                const int sgi = mb.molmon[k];
                double nmon = 0;
                for (auto& B : mb.blocks) if (B.seg == sgi) nmon += B.length * B.degeneracy;
                if (H->seg_nstate[sgi] > 0) {
                    for (int j = 0; j < P.n_state; j++)
                        if (H->state_seg[j] == sgi) q += H->state_alphabulk[j] * H->state_valence[j] * nmon;
                } else q += H->seg_valence[sgi] * nmon;
            }
            mb.mol.charge = q / N;
        }
        if (mb.mol.freedom == NM_MOL_RESTRICTED) {
            bool hn = in.has("mol", mn, "n"), ht = in.has("mol", mn, "theta");
            if (hn == ht) { err = "restricted mol " + mn + " needs exactly one of n / theta"; delete H; return nullptr; }
            if (hn) { to_real(in.get("mol", mn, "n"), mb.mol.n); mb.mol.theta = mb.mol.n * N; }
            else { to_real(in.get("mol", mn, "theta"), mb.mol.theta); mb.mol.n = mb.mol.theta / N; }
        }
        if (mb.mol.pinned && mb.mol.freedom != NM_MOL_RESTRICTED) {
            err = "mol " + mn + " with a pinned segment must be restricted"; delete H; return nullptr;
        }
        mb.mol.n_molmon = (int)mb.molmon.size();
        mb.mol.n_blocks = (int)mb.blocks.size();
        mb.mol.n_store = mb.n_store;
        // Markov 2: semiflexible chains (molecule.cpp:627-674), the bond-angle
        // weights of Molecule::AllocateMemory (molecule.cpp:135-152): FJC = 3
        // directions on a simple-cubic lattice, P[k] = exp(-k_stiff/2·(kπ/2)²)
        // for k = 0, 1 over Q = P[0] + 4·P[1], P[2] = 0
        mb.mol.markov = 1;
        if (in.has("mol", mn, "Markov")) {
            int mk = 0;
            if (!to_int(in.get("mol", mn, "Markov"), mk) || mk < 1 || mk > 2) {
                err = "mol " + mn + ": Markov is 1 or 2"; delete H; return nullptr;
            }
            mb.mol.markov = mk;
        }
        if (mb.mol.markov == 2) {
            std::string why;
            if (P.gradients != 1) why = "1-gradient lattices";
            else if (P.lattice_type != NM_SIMPLE_CUBIC) why = "simple-cubic lattices";
            else if (mb.is_dendrimer || comp.find('[') != std::string::npos) why = "linear chains";
            if (!why.empty()) {
                err = "mol " + mn + ": Markov 2 is built for " + why + " only"; delete H; return nullptr;
            }
            // the reference's default is the lattice's k_stiff, which it never sets
            if (!in.has("mol", mn, "k_stiff")) {
                err = "mol " + mn + ": Markov 2 needs k_stiff"; delete H; return nullptr;
            }
            double ks = 0;
            if (!to_real(in.get("mol", mn, "k_stiff"), ks) || ks < 0 || ks > 10) {
                err = "mol " + mn + ": k_stiff in [0, 10]"; delete H; return nullptr;
            }
            const int FJC = 3;
            double Pk[FJC], Q = 0;
            for (int k = 0; k < FJC - 1; k++) {
                const double a = k * PIE / (FJC - 1);
                Pk[k] = std::exp(-0.5 * ks * a * a);
                if (k > 0) Q += 4 * Pk[k];
                else Q = Pk[k];
            }
            Pk[FJC - 1] = 0;
            for (int k = 0; k < FJC; k++) mb.mol.bend[k] = Pk[k] / Q;
        } else if (in.has("mol", mn, "k_stiff")) {
            // read, range-checked and unused with Markov 1 (molecule.cpp:634-641)
            double ks = 0;
            if (!to_real(in.get("mol", mn, "k_stiff"), ks) || ks < 0 || ks > 10) {
                err = "mol " + mn + ": k_stiff in [0, 10]"; delete H; return nullptr;
            }
        }
    }
    // solvent rules (system.cpp CheckInput)
    if (P.solvent < 0) {
        if (!(nmol == 1 && H->mb[0].mol.pinned)) { err = "one molecule must have freedom : solvent"; delete H; return nullptr; }
    }
    // ---- iteration list (MakeItsLists / IsUnique, system.cpp:430-500, 1218+) ----
    // A segment or state whose χ row equals an earlier block's
    // representative's shares that block.  Segments with states are not
    // blocks themselves; ItStateList follows ItMonList.
    const int nsp = P.n_state > 0 ? P.n_sp : ns;
    const double* chi_rows = P.n_state > 0 ? H->chi_sp.data() : H->chi.data();
    auto same_row = [&](int a, int b) {
        for (int k = 0; k < nsp; k++) if (chi_rows[(size_t)a * nsp + k] != chi_rows[(size_t)b * nsp + k]) return false;
        return true;
    };
    H->seg_it.assign(ns, -1);
    std::vector<int> sysmon;
    for (int m = 0; m < nmol; m++)
        for (int sgi : H->mb[m].molmon) {
            if (std::find(sysmon.begin(), sysmon.end(), sgi) != sysmon.end()) continue;
            sysmon.push_back(sgi);
            if (H->seg_nstate[sgi] > 0) continue;
            int copy_of = -1;
            for (size_t j = 0; j < H->it_sp.size() && copy_of < 0; j++)
                if (same_row(sgi, H->it_sp[j])) copy_of = (int)j;
            if (copy_of < 0) { H->seg_it[sgi] = (int)H->it_sp.size(); H->it_sp.push_back(sgi); H->it_seg.push_back(sgi); }
            else H->seg_it[sgi] = copy_of;
        }
    H->state_it.assign(P.n_state, -1);
    for (int j = 0; j < P.n_state; j++) {
        int copy_of = -1;
        for (size_t b = 0; b < H->it_sp.size() && copy_of < 0; b++)
            if (same_row(ns + j, H->it_sp[b])) copy_of = (int)b;
        if (copy_of < 0) {
            H->state_it[j] = (int)H->it_sp.size();
            H->it_sp.push_back(ns + j);
            H->it_seg.push_back(H->state_seg[j]);
        } else H->state_it[j] = copy_of;
    }
    P.n_it = (int)H->it_seg.size();
    P.charged = 0;
    for (int i = 0; i < ns; i++) if (H->seg_valence[i] != 0) P.charged = 1;
    for (int j = 0; j < P.n_state; j++) if (H->state_valence[j] != 0) P.charged = 1;
    if (P.n_state > 0 && P.n_sp > 16) {
        err = "more than 16 interaction species (mons without states, and states)"; delete H; return nullptr;
    }
    for (int m = 0; m < nmol; m++) {
        if (H->mb[m].mol.markov != 2) continue;
        if (P.charged) { err = "Markov 2 chains in a charged system are not built"; delete H; return nullptr; }
        for (int sgi : H->mb[m].molmon)
            if (H->seg_nstate[sgi] > 0) {
                err = "Markov 2 chains with internal states are not built"; delete H; return nullptr;
            }
    }
    P.iv = P.n_it * M + (P.charged ? M : 0);
    // ---- newton ----
    auto newt = in.order("newton");
    P.diis_m = 10; P.iterationlimit = 1000; P.tolerance = 1e-7; P.deltamax = 0.1; P.max_norm = 0;
    if (!newt.empty()) {
        const std::string& nn = newt[0];
        std::string meth = in.get("newton", nn, "method", "DIIS");
        if (meth != "DIIS") H->method_note = "newton method '" + meth + "' replaced by DIIS";
        double v; int iv;
        if (in.has("newton", nn, "tolerance") && to_real(in.get("newton", nn, "tolerance"), v)) P.tolerance = v;
        if (in.has("newton", nn, "deltamax") && to_real(in.get("newton", nn, "deltamax"), v)) P.deltamax = v;
        if (in.has("newton", nn, "m") && to_int(in.get("newton", nn, "m"), iv)) P.diis_m = iv;
        if (in.has("newton", nn, "iterationlimit") && to_int(in.get("newton", nn, "iterationlimit"), iv)) P.iterationlimit = iv;
        if (in.get("newton", nn, "stop_criterion") == "max_of_element_of_|g|") P.max_norm = 1;
        if (P.diis_m < 1 || P.diis_m > 100) P.diis_m = 10;
        if (P.iterationlimit < 0 || P.iterationlimit > 1000000) P.iterationlimit = 1000;
    }
    // the outer (search) iteration's controls, defaults of solve_scf.cpp:153-177
    P.super_tolerance = 10.0 * P.tolerance;
    P.super_iterationlimit = P.iterationlimit / 10;
    P.super_deltamax = 0.5;
    if (!newt.empty()) {
        const std::string& nn = newt[0];
        double v; int iv;
        if (in.has("newton", nn, "super_tolerance") && to_real(in.get("newton", nn, "super_tolerance"), v))
            P.super_tolerance = v;
        if (in.has("newton", nn, "super_iterationlimit") && to_int(in.get("newton", nn, "super_iterationlimit"), iv))
            P.super_iterationlimit = iv;
        if (in.has("newton", nn, "super_deltamax") && to_real(in.get("newton", nn, "super_deltamax"), v))
            P.super_deltamax = v;
    }
    // ---- a search: `var : mol-<name> : search : theta|n|phibulk` and one
    // target, `var : sys-<name> : free_energy|grand_potential : <value>` or
    // `var : mol-<name> : theta|n|phibulk|mu : <value>` (Variate::CheckInput,
    // variate.cpp:60-200; Molecule::PutVarInfo, molecule.cpp:679-740) ----
    P.scan_mol = -1; P.scan_what = -1; P.scan_n = 0; P.scan_exponential = 0; P.scan_state = -1;
    P.scan_reaction = -1;
    P.scan_start = P.scan_end = P.scan_step = 0;
    P.search_mol = -1; P.search_what = -1;
    P.target_kind = -1; P.target_mol = -1; P.target_what = -1; P.target_value = 0;
    {
        static const char* const what[] = {"theta", "n", "phibulk", "mu"};
        for (const std::string& vn : in.order("var")) {
            const size_t dash = vn.find('-');
            if (dash == std::string::npos || vn.find('-', dash + 1) != std::string::npos) {
                err = "var '" + vn + "': the name is <item>-<name>, e.g. mol-pol";
                delete H; return nullptr;
            }
            const std::string item = vn.substr(0, dash), name = vn.substr(dash + 1);
            auto set_target = [&](int kind, int mol, int w, const std::string& val) {
                if (P.target_kind >= 0) { err = "a search takes one target"; return false; }
                double t;
                if (!to_real(val, t)) { err = "var '" + vn + "': the target value '" + val + "' is not a number"; return false; }
                P.target_kind = kind; P.target_mol = mol; P.target_what = w; P.target_value = t;
                return true;
            };
            if (item == "mol") {
                int mi = -1;
                for (int m = 0; m < nmol; m++) if (molnames[m] == name) mi = m;
                if (mi < 0) { err = "var '" + vn + "': no molecule " + name; delete H; return nullptr; }
                if (in.has("var", vn, "search")) {
                    const std::string sv = in.get("var", vn, "search");
                    int w = -1;
                    for (int k = 0; k < 3; k++) if (sv == what[k]) w = k;
                    if (w < 0) { err = "var '" + vn + "': search takes theta, n or phibulk"; delete H; return nullptr; }
                    if (P.search_mol >= 0) { err = "one search per input"; delete H; return nullptr; }
                    const int fr = H->mb[mi].mol.freedom;
                    if ((w < 2 && fr != NM_MOL_RESTRICTED) || (w == 2 && fr != NM_MOL_FREE)) {
                        err = "var '" + vn + "': theta and n are searched on a restricted molecule, phibulk on a free one";
                        delete H; return nullptr;
                    }
                    P.search_mol = mi; P.search_what = w;
                }
                for (int k = 0; k < 4; k++)
                    if (in.has("var", vn, what[k]) && !set_target(2, mi, k, in.get("var", vn, what[k]))) {
                        delete H; return nullptr;
                    }
                if (in.has("var", vn, "scan")) {
                    // Variate::CheckInput (variate.cpp:280-336), Molecule::PutVarScan
                    const std::string sv = in.get("var", vn, "scan");
                    int w = -1;
                    for (int k = 0; k < 3; k++) if (sv == what[k]) w = k;
                    const nm_molecule& mol = H->mb[mi].mol;
                    const bool fits = (w < 2 && mol.freedom == NM_MOL_RESTRICTED) || (w == 2 && mol.freedom == NM_MOL_FREE);
                    if (w < 0 || !fits) {
                        err = "var '" + vn + "': scan takes theta or n of a restricted molecule, phibulk of a free one";
                        delete H; return nullptr;
                    }
                    if (P.scan_mol >= 0) { err = "one scan per input"; delete H; return nullptr; }
                    double end = 0, step = 0;
                    if (!in.has("var", vn, "end_value") || !to_real(in.get("var", vn, "end_value"), end)) {
                        err = "var '" + vn + "': a scan needs a numeric end_value"; delete H; return nullptr;
                    }
                    const std::string scale = in.get("var", vn, "scale", "linear");
                    const double start = w == 0 ? mol.theta : w == 1 ? mol.n : mol.phibulk;
                    int nsteps = 0;
                    if (scale == "exponential") {
                        int steps = 1;
                        if (in.has("var", vn, "steps") && (!to_int(in.get("var", vn, "steps"), steps) || steps < 1)) {
                            err = "var '" + vn + "': steps (per decade) must be a positive integer"; delete H; return nullptr;
                        }
                        if (!(end > 0 && start > 0)) {
                            err = "var '" + vn + "': an exponential scan needs a positive start and end_value";
                            delete H; return nullptr;
                        }
                        const double ns_real = end > start ? steps * std::log10(end / start) : steps * std::log10(start / end);
                        if (!(ns_real < 1e6)) { err = "var '" + vn + "': more than 10^6 scan steps"; delete H; return nullptr; }
                        nsteps = (int)ns_real;
                        P.scan_exponential = 1;
                    } else if (scale == "linear") {
                        if (!in.has("var", vn, "step") || !to_real(in.get("var", vn, "step"), step) || step == 0) {
                            err = "var '" + vn + "': a linear scan needs a nonzero step"; delete H; return nullptr;
                        }
                        // the step count is (end - start)/step truncated to an
                        // int first, as the reference assigns it
                        // (molecule.cpp:807-812): a ratio in (-1, 0) is a
                        // zero-step scan, a truncated count below 0 is refused
                        const double ns_real = (end - start) / step;
                        if (!(ns_real < 1e6 && ns_real > -1e6)) {
                            err = "var '" + vn + "': more than 10^6 scan steps"; delete H; return nullptr;
                        }
                        nsteps = (int)ns_real;
                        if (nsteps < 0) {
                            err = "var '" + vn + "': (end_value - start)/step is negative"; delete H; return nullptr;
                        }
                    } else {
                        err = "var '" + vn + "': scale is linear or exponential"; delete H; return nullptr;
                    }
                    P.scan_mol = mi; P.scan_what = w; P.scan_n = nsteps;
                    P.scan_start = start; P.scan_end = end; P.scan_step = step;
                }
            } else if (item == "state" && in.has("var", vn, "scan")) {
                // a fixed state's bulk fraction (State::PutVarInfo / PutVarScan,
                // state.cpp:229-304): the same step rules as a molecule's scan
                int sj = -1;
                for (int j = 0; j < P.n_state; j++) if (H->state_names[j] == name) sj = j;
                if (sj < 0) { err = "var '" + vn + "': no state " + name; delete H; return nullptr; }
                if (in.get("var", vn, "scan") != "alphabulk" || !H->state_fixed[sj]) {
                    err = "var '" + vn + "': a state scan takes the alphabulk of a state that fixes it";
                    delete H; return nullptr;
                }
                if (P.scan_mol >= 0 || P.scan_state >= 0 || P.scan_reaction >= 0) {
                    err = "one scan per input"; delete H; return nullptr;
                }
                double end = 0, step = 0;
                if (!in.has("var", vn, "end_value") || !to_real(in.get("var", vn, "end_value"), end)) {
                    err = "var '" + vn + "': a scan needs a numeric end_value"; delete H; return nullptr;
                }
                const std::string scale = in.get("var", vn, "scale", "linear");
                const double start = H->state_ab_in[sj];
                int nsteps = 0;
                if (scale == "exponential") {
                    int steps = 1;
                    if (in.has("var", vn, "steps") && (!to_int(in.get("var", vn, "steps"), steps) || steps < 1)) {
                        err = "var '" + vn + "': steps (per decade) must be a positive integer"; delete H; return nullptr;
                    }
                    if (!(end > 0 && start > 0)) {
                        err = "var '" + vn + "': an exponential scan needs a positive start and end_value";
                        delete H; return nullptr;
                    }
                    const double ns_real = end > start ? steps * std::log10(end / start) : steps * std::log10(start / end);
                    if (!(ns_real < 1e6)) { err = "var '" + vn + "': more than 10^6 scan steps"; delete H; return nullptr; }
                    nsteps = (int)ns_real;
                    P.scan_exponential = 1;
                } else if (scale == "linear") {
                    if (!in.has("var", vn, "step") || !to_real(in.get("var", vn, "step"), step) || step == 0) {
                        err = "var '" + vn + "': a linear scan needs a nonzero step"; delete H; return nullptr;
                    }
                    const double ns_real = (end - start) / step;
                    if (!(ns_real < 1e6 && ns_real > -1e6)) {
                        err = "var '" + vn + "': more than 10^6 scan steps"; delete H; return nullptr;
                    }
                    nsteps = (int)ns_real;
                    if (nsteps < 0) { err = "var '" + vn + "': (end_value - start)/step is negative"; delete H; return nullptr; }
                } else {
                    err = "var '" + vn + "': scale is linear or exponential"; delete H; return nullptr;
                }
                P.scan_state = sj; P.scan_what = 3; P.scan_n = nsteps;
                P.scan_start = start; P.scan_end = end; P.scan_step = step;
            } else if (item == "reaction" && in.has("var", vn, "scan")) {
                // a reaction's pK, linear steps only (Reaction::PutVarInfo /
                // PutVarScan, reaction.cpp:381-408)
                int ri = -1;
                for (size_t r = 0; r < H->reactions.size(); r++) if (H->reactions[r].name == name) ri = (int)r;
                if (ri < 0) { err = "var '" + vn + "': no reaction " + name; delete H; return nullptr; }
                if (in.get("var", vn, "scan") != "pK") { err = "var '" + vn + "': a reaction scan takes pK"; delete H; return nullptr; }
                if (P.scan_mol >= 0 || P.scan_state >= 0 || P.scan_reaction >= 0) {
                    err = "one scan per input"; delete H; return nullptr;
                }
                if (in.get("var", vn, "scale", "linear") != "linear") {
                    err = "var '" + vn + "': a pK scan is linear"; delete H; return nullptr;
                }
                double end = 0, step = 0;
                if (!in.has("var", vn, "end_value") || !to_real(in.get("var", vn, "end_value"), end)) {
                    err = "var '" + vn + "': a scan needs a numeric end_value"; delete H; return nullptr;
                }
                if (!in.has("var", vn, "step") || !to_real(in.get("var", vn, "step"), step) || step == 0) {
                    err = "var '" + vn + "': a linear scan needs a nonzero step"; delete H; return nullptr;
                }
                const double start = H->reactions[ri].pK;
                const double ns_real = (end - start) / step;
                if (!(ns_real < 1e6 && ns_real > -1e6)) { err = "var '" + vn + "': more than 10^6 scan steps"; delete H; return nullptr; }
                const int nsteps = (int)ns_real;
                if (nsteps < 0) { err = "var '" + vn + "': (end_value - start)/step is negative"; delete H; return nullptr; }
                P.scan_reaction = ri; P.scan_what = 4; P.scan_n = nsteps;
                P.scan_start = start; P.scan_end = end; P.scan_step = step;
            } else if (item == "sys") {
                if (in.has("var", vn, "free_energy") && !set_target(0, -1, -1, in.get("var", vn, "free_energy"))) {
                    delete H; return nullptr;
                }
                if (in.has("var", vn, "grand_potential") &&
                    !set_target(1, -1, -1, in.get("var", vn, "grand_potential"))) {
                    delete H; return nullptr;
                }
            }
        }
        if ((P.search_mol >= 0) != (P.target_kind >= 0)) {
            err = "a search needs one 'search' and one target";
            delete H; return nullptr;
        }
        // the reference's search solves the bulk equilibrium again before
        // each inner solve (Solve_scf::residuals -> Solve, solve_scf.cpp:848),
        // from the previous inner solve's bulk fractions; not restated
        if (P.search_mol >= 0 && P.n_state > 0) {
            err = "a search on a system with internal states is not supported";
            delete H; return nullptr;
        }
        // a free molecule's θ or n as the target: the reference's run of
        // such a search (φ_bulk of an adsorbing free polymer for a target θ)
        // ends in NaN, so it is refused rather than run
        if (P.target_kind == 2 && P.target_what <= 1 && H->mb[P.target_mol].mol.freedom == NM_MOL_FREE) {
            err = "a search for a free molecule's theta or n is not supported (the reference's ends in NaN)";
            delete H; return nullptr;
        }
    }
    // ---- publish pointers ----
    for (auto& s : H->seg_names) H->seg_name_ptrs.push_back(s.c_str());
    P.seg_name = H->seg_name_ptrs.data();
    P.seg_freedom = H->seg_freedom.data();
    P.seg_it = H->seg_it.data();
    P.seg_gmask = H->seg_gmask.data();
    P.seg_phi_frozen = H->seg_phi_frozen.data();
    P.chi = H->chi.data();
    P.seg_valence = H->seg_valence.data();
    P.seg_epsilon = H->seg_epsilon.data();
    P.ksam = H->ksam.data();
    P.it_seg = H->it_seg.data();
    if (P.n_state > 0) {
        for (auto& s : H->state_names) H->state_name_ptrs.push_back(s.c_str());
        P.state_name = H->state_name_ptrs.data();
        P.state_seg = H->state_seg.data();
        P.state_valence = H->state_valence.data();
        P.state_alphabulk = H->state_alphabulk.data();
        P.state_it = H->state_it.data();
        P.seg_nstate = H->seg_nstate.data();
        P.chi_sp = H->chi_sp.data();
        P.it_sp = H->it_sp.data();
    } else {
        P.n_sp = ns;
    }
    H->mols.resize(nmol);
    for (int m = 0; m < nmol; m++) {
        MolBuild& mb = H->mb[m];
        mb.mol.molmon_seg = mb.molmon.data();
        mb.mol.molmon_fraction = mb.fraction.data();
        mb.mol.blocks = mb.blocks.data();
        mb.mol.child_index = mb.child_index.data();
        H->mols[m] = mb.mol;
    }
    P.n_mol = nmol;
    P.mols = H->mols.data();
    H->mol_names.assign(molnames.begin(), molnames.end());
    for (auto& s : H->mol_names) H->mol_name_ptrs.push_back(s.c_str());
    P.mol_name = H->mol_name_ptrs.data();
    return &H->plan;
}

}  // namespace nm

extern "C" {

int nm_plan_create(const char* input_text, nm_plan** out) {
    if (!input_text || !out) { nm::set_error("nm_plan_create: null argument"); return NM_ERR_ARG; }
    *out = nullptr;
    nm::InputBlock blk;
    if (!nm::parse_input(input_text, blk)) return NM_ERR_INPUT;
    std::string err;
    nm_plan* p = nm::build_plan(blk, err);
    if (!p) { nm::set_error(err); return NM_ERR_INPUT; }
    if (!nm::check_unread(blk, err)) {
        nm_plan_destroy(p);
        nm::set_error(err);
        return NM_ERR_INPUT;
    }
    *out = p;
    return NM_OK;
}

int nm_plan_state_bulk(const nm_plan* plan, const double* fixed_ab, const double* pK, const double* sp_phibulk,
                       double* alphabulk, double* mol_charge) {
    if (!plan || plan->n_state == 0) { nm::set_error("nm_plan_state_bulk: the plan has no internal states"); return NM_ERR_ARG; }
    const nm::PlanHolder& H = *reinterpret_cast<const nm::PlanHolder*>(plan);
    std::vector<double> fx = fixed_ab ? std::vector<double>(fixed_ab, fixed_ab + plan->n_state) : H.state_ab_in;
    std::vector<double> pk = nm::plan_reaction_pK(plan);
    if (pK) pk.assign(pK, pK + pk.size());
    std::vector<double> ab, q;
    std::string err;
    if (int rc = nm::plan_state_bulk(plan, fx, pk, sp_phibulk, ab, q, err)) { nm::set_error("nm_plan_state_bulk: " + err); return rc; }
    if (alphabulk) std::copy(ab.begin(), ab.end(), alphabulk);
    if (mol_charge) std::copy(q.begin(), q.end(), mol_charge);
    return NM_OK;
}

int nm_plan_scan_value(const nm_plan* plan, int k, double* value) {
    if (!plan || !value || (plan->scan_mol < 0 && plan->scan_state < 0 && plan->scan_reaction < 0) || k < 0 ||
        k > plan->scan_n) {
        nm::set_error("nm_plan_scan_value: no scan, or step out of range");
        return NM_ERR_ARG;
    }
    const double a = plan->scan_start, b = plan->scan_end;
    if (!plan->scan_exponential) *value = a + k * plan->scan_step;
    else if (plan->scan_n == 0) *value = a;
    else {
        const double f = 1.0 * k / plan->scan_n;
        *value = std::pow(10.0, (1 - f) * std::log10(a) + f * std::log10(b));
    }
    return NM_OK;
}

void nm_plan_destroy(nm_plan* plan) {
    if (plan) delete reinterpret_cast<nm::PlanHolder*>(plan);
}

const char* nm_last_error(void) { return nm::g_last_error.c_str(); }

const char* nm_version(void) { return "namics_gb300 0.1 (sm_103a)"; }

}  // extern "C"

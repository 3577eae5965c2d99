// Randomised check of constant folding (fold_program): random Solid trees are
// lowered, random leaves marked inactive (false) and random leaf values drawn;
// the folded program must evaluate like the full one.  Host logic only.
#include "../../model3d_gb300/csrc/mc_lower.h"
#include <cstdio>
#include <random>
using namespace mcgpu;
// Reference evaluation of a postfix program given leaf values (no transforms; boxes = given bits)
static int eval(const uint32_t* q, int n, const std::vector<int>& lv, const std::vector<int>& box) {
    std::vector<int> st;
    for (int i = 0; i < n; i++) {
        uint32_t op = q[i], c = op_code(op), a = op_arg(op);
        switch (c) {
            case OP_LEAF: st.push_back(lv[a]); break;
            case OP_JLEAVES: { int v = 0; for (uint32_t l = range_first(a); l < range_first(a) + range_count(a); l++) v |= lv[l]; st.push_back(v); break; }
            case OP_ALEAVES: { int v = 1; for (uint32_t l = range_first(a); l < range_first(a) + range_count(a); l++) v &= lv[l]; st.push_back(v); break; }
            case OP_JLIST: { int v = 0; for (uint32_t k = 0; k < a; k++) v |= lv[q[i + 1 + k]]; i += a; st.push_back(v); break; }
            case OP_OR: { int b = st.back(); st.pop_back(); st.back() |= b; break; }
            case OP_AND: { int b = st.back(); st.pop_back(); st.back() &= b; break; }
            case OP_ANDNOT: { int b = st.back(); st.pop_back(); st.back() &= !b; break; }
            case OP_NOT: st.back() = !st.back(); break;
            case OP_BOX: st.push_back(box[a]); break;
            case OP_BOXAND: st.back() &= box[a]; break;
            case OP_TRUE: st.push_back(1); break;
            case OP_FALSE: st.push_back(0); break;
            default: printf("bad op %u\n", c); return -1;
        }
    }
    return st.empty() ? 0 : st[0];
}
std::mt19937 rng(1);
// random tree as mc_node prefix records
static void gen(std::vector<mc_node>& out, int depth) {
    mc_node n{}; 
    int r = rng() % 10;
    if (depth == 0 || r < 4) { n.kind = MC_NODE_SPHERE; n.p[3] = 0.5; for (int i=0;i<3;i++){n.min[i]=-1;n.max[i]=1;} out.push_back(n); return; }
    for (int i=0;i<3;i++){n.min[i]=-1;n.max[i]=1;}
    if (r < 6) { n.kind = MC_NODE_JOIN; n.n_children = 1 + rng() % 6; out.push_back(n); for (int i = 0; i < n.n_children; i++) gen(out, depth - 1); }
    else if (r < 7) { n.kind = MC_NODE_INTERSECT; n.n_children = 1 + rng() % 4; out.push_back(n); for (int i = 0; i < n.n_children; i++) gen(out, depth - 1); }
    else if (r < 9) { n.kind = MC_NODE_SUBTRACT; n.n_children = 2; out.push_back(n); gen(out, depth - 1); gen(out, depth - 1); }
    else { n.kind = MC_NODE_CHECKED; n.n_children = 1; out.push_back(n); gen(out, depth - 1); }
}
int main() {
    int bad = 0, trials = 0;
    for (int t = 0; t < 3000; t++) {
        std::vector<mc_node> nodes; gen(nodes, 4);
        HostProgram P; lower_scene(nodes.data(), nodes.size(), nullptr, 0, &P);
        int L = P.leaf_kind.size(), B = P.xbox.size();
        std::vector<uint32_t> q(P.fold_cap + 1);
        for (int k = 0; k < 20; k++) {
            std::vector<uint32_t> act((L + 31) / 32, 0);
            std::vector<int> lv(L), box(B);
            for (int l = 0; l < L; l++) { if (rng() % 2) act[l >> 5] |= 1u << (l & 31); lv[l] = (act[l>>5] >> (l&31) & 1) ? (int)(rng() % 2) : 0; }
            for (int b = 0; b < B; b++) box[b] = rng() % 2;
            int full = eval(P.ops.data(), P.ops.size(), lv, box);
            int n = fold_program(P.ops.data(), P.ops.size(), act.data(), q.data());
            if (n > P.fold_cap) { printf("overflow\n"); bad++; }
            int f = n == FOLD_FALSE ? 0 : n == FOLD_TRUE ? 1 : eval(q.data(), n, lv, box);
            trials++;
            if (f != full) { bad++; if (bad < 5) printf("mismatch t=%d k=%d full=%d folded=%d n=%d ops=%zu\n", t, k, full, f, n, P.ops.size()); }
        }
        // all-false fold from the host
        std::vector<int> lv0(L, 0), box(B); for (int b = 0; b < B; b++) box[b] = rng() % 2;
        int full = eval(P.ops.data(), P.ops.size(), lv0, box);
        int n = P.n_ops_allfalse;
        int f = n == FOLD_FALSE ? 0 : n == FOLD_TRUE ? 1 : eval(P.ops_allfalse.data(), n, lv0, box);
        if (f != full) { bad++; printf("allfalse mismatch\n"); }
    }
    printf("trials %d bad %d\n", trials, bad);
    return bad != 0;
}

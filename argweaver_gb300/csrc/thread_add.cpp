// Adding a sampled thread to the ARG (add_arg_thread, thread.cpp:272-422), on the host:
// the new leaf joins every local tree at the state its thread takes at the tree's first
// column, each sampled recombination splits its tree in two by an SPR, and the node
// mappings and SPRs between neighbouring trees are renamed for the two new nodes
// (add_spr_branch, thread.cpp:176-269). Pointer surgery on a few hundred nodes per tree:
// host work between the device's threading passes.
//
// Node names follow the reference: the new leaf takes the name nleaves, the node that had
// it moves to nnodes (displaced), the new coalescence node is nnodes + 1. Child order is
// kept as the reference keeps it (it decides which child a later SPR replaces), so the
// handle stores children next to parents.

#include <cstring>
#include <string>
#include <vector>

#include "thread_add.h"

namespace awg {

namespace {

struct Node {
    int parent = -1, c0 = -1, c1 = -1, age = 0;
};

struct Tree {
    std::vector<Node> nd;
    int root = -1;
};

// rename_node (thread.cpp:9-36): node src moves to dest, its neighbours follow
void rename_node(Tree &t, int src, int dest) {
    if (src == dest) return;
    t.nd[dest] = t.nd[src];
    const int parent = t.nd[dest].parent;
    if (parent != -1) {
        if (t.nd[parent].c0 == src) t.nd[parent].c0 = dest;
        else t.nd[parent].c1 = dest;
    }
    if (t.nd[dest].c0 != -1) t.nd[t.nd[dest].c0].parent = dest;
    if (t.nd[dest].c1 != -1) t.nd[t.nd[dest].c1].parent = dest;
}

// add_tree_branch (thread.cpp:39-101): the new leaf coalesces at (node, time)
void add_tree_branch(Tree &t, int nnodes, int node, int time) {
    const int nleaves = (nnodes + 1) / 2;
    const int newleaf = nleaves, displaced = nnodes, newcoal = nnodes + 1;
    t.nd.resize(nnodes + 2);
    const int node2 = node != newleaf ? node : displaced;
    const int parent = t.nd[node].parent;
    const int parent2 = parent != newleaf ? parent : displaced;
    if (newleaf < displaced) rename_node(t, newleaf, displaced);
    t.nd[newleaf] = Node{newcoal, -1, -1, 0};
    t.nd[newcoal] = Node{parent2, newleaf, node2, time};
    t.nd[node2].parent = newcoal;
    if (parent2 != -1) {
        if (t.nd[parent2].c0 == node2) t.nd[parent2].c0 = newcoal;
        else t.nd[parent2].c1 = newcoal;
    }
    if (t.nd[newcoal].parent == -1) t.root = newcoal;
    else t.root = t.root != newleaf ? t.root : displaced;
}

// apply_spr (local_tree.cpp:223-313)
void apply_spr(Tree &t, const int spr[4]) {
    const int rnode = spr[0], cnode = spr[2];
    if (rnode == t.root) return;
    const int recoal = t.nd[rnode].parent;
    const int other = t.nd[recoal].c0 == rnode ? 1 : 0;
    const int recomb_sib = other ? t.nd[recoal].c1 : t.nd[recoal].c0;
    const int broke_parent = t.nd[recoal].parent;
    auto child = [&](int v, int x) -> int & { return x ? t.nd[v].c1 : t.nd[v].c0; };
    t.nd[recomb_sib].parent = broke_parent;
    int x = 0;
    if (broke_parent != -1) {
        x = t.nd[broke_parent].c0 == recoal ? 0 : 1;
        child(broke_parent, x) = recomb_sib;
    }
    if (cnode == recoal) {
        child(recoal, other) = recomb_sib;
        t.nd[recoal].parent = t.nd[recomb_sib].parent;
        t.nd[recomb_sib].parent = recoal;
        if (broke_parent != -1) child(broke_parent, x) = recoal;
    } else {
        child(recoal, other) = cnode;
        t.nd[recoal].parent = t.nd[cnode].parent;
        t.nd[cnode].parent = recoal;
        const int parent = t.nd[recoal].parent;
        if (parent != -1) {
            if (t.nd[parent].c0 == cnode) t.nd[parent].c0 = recoal;
            else t.nd[parent].c1 = recoal;
        }
    }
    t.nd[recoal].age = spr[3];
    int root;
    if (cnode == t.root) root = recoal;
    else if (recoal == t.root) root = cnode == recomb_sib ? recoal : recomb_sib;
    else root = t.root;
    t.root = root;
}

// state k of an external tree (get_coal_states_external, states.cpp:53-74)
bool state_of(const Tree &t, int nnodes, int T, int k, int &node, int &time) {
    if (k < 0) return false;
    for (int v = 0; v < nnodes; v++) {
        const int top = t.nd[v].parent == -1 ? T - 2 : t.nd[t.nd[v].parent].age;
        const int m = top - t.nd[v].age + 1;
        if (m <= 0) continue;
        if (k < m) {
            node = v;
            time = t.nd[v].age + k;
            return true;
        }
        k -= m;
    }
    return false;
}

// add_spr_branch (thread.cpp:176-269): the SPR into `t` and its mapping renamed for the
// new leaf and coalescence node
bool add_spr_branch(const Tree &t, const Tree &last, int state_node, int state_time,
                    int last_node, int *spr, std::vector<int> &mapping, int newleaf,
                    int displaced, int newcoal, int nnodes2) {
    const int last_node2 = last_node != newleaf ? last_node : displaced;
    const int node2 = state_node != newleaf ? state_node : displaced;
    mapping[displaced] = mapping[newleaf];
    mapping[newleaf] = newleaf;
    mapping[newcoal] = newcoal;
    for (int i = newleaf + 1; i < nnodes2; i++)
        if (mapping[i] == newleaf) mapping[i] = displaced;
    if (spr[0] == newleaf) spr[0] = displaced;
    if (spr[2] == newleaf) spr[2] = displaced;
    if (mapping[spr[0]] < 0) return false;
    const int recoal = t.nd[mapping[spr[0]]].parent;
    if (recoal == newcoal) {
        if (mapping[last_node2] == node2) {
            spr[0] = newcoal;  // recombination above the coalescence state: renamed
        } else {
            const int sn = state_node != newleaf ? state_node : displaced;
            if (sn == mapping[spr[0]]) {  // mediated coalescence
                spr[2] = newleaf;
                spr[3] = state_time;
            }  // else the new branch escapes: nothing to rename
        }
    } else if (recoal != -1 && (t.nd[recoal].c0 == newcoal || t.nd[recoal].c1 == newcoal)) {
        if (last.nd[spr[2]].parent == newcoal) spr[2] = newcoal;
    }
    if (last.nd[spr[0]].parent == newcoal) {  // newcoal was the broken node
        mapping[newcoal] = -1;
        const int p = last.nd[newcoal].parent;
        if (p != -1) mapping[p] = newcoal;
    } else {  // follow a child without the recombination or coalescence down to a mapped node
        int x = newcoal;
        for (int steps = 0;; steps++) {
            if (steps > nnodes2) return false;
            int y = last.nd[x].c0;
            if (y == spr[2] || y == spr[0]) y = last.nd[x].c1;
            x = y;
            if (x < 0) return false;
            if (mapping[x] != -1) break;
        }
        mapping[newcoal] = t.nd[mapping[x]].parent;
    }
    return true;
}

}  // namespace

bool add_arg_thread(ThreadTrees &a, int T, const int *path, int seqlen, const int *rec_pos,
                    const int *rec_node, const int *rec_time, int nrec, std::string &err) {
    const int nnodes = a.nnodes, nnodes2 = nnodes + 2, B = a.ntrees;
    const int nleaves = (nnodes + 1) / 2;
    const int newleaf = nleaves, displaced = nnodes, newcoal = nnodes + 1;
    long long total = 0;
    for (int b = 0; b < B; b++) total += a.blocklens[b];
    if (total != seqlen) {
        err = "add_arg_thread: the path does not cover the trees";
        return false;
    }
    for (int r = 0; r < nrec; r++)
        if (rec_pos[r] <= 0 || rec_pos[r] >= seqlen || (r > 0 && rec_pos[r] <= rec_pos[r - 1])) {
            err = "add_arg_thread: recombination columns must increase within the region";
            return false;
        }
    // the input trees, children as stored (index order unless the handle kept an order)
    std::vector<Tree> in(B);
    for (int b = 0; b < B; b++) {
        Tree &t = in[b];
        t.nd.resize(nnodes);
        for (int i = 0; i < nnodes; i++) {
            t.nd[i].parent = a.ptrees[(size_t)b * nnodes + i];
            t.nd[i].age = a.ages[(size_t)b * nnodes + i];
            if (t.nd[i].parent == -1) t.root = i;
        }
        if (!a.c0.empty()) {
            for (int i = 0; i < nnodes; i++) {
                t.nd[i].c0 = a.c0[(size_t)b * nnodes + i];
                t.nd[i].c1 = a.c1[(size_t)b * nnodes + i];
            }
        } else {
            for (int i = 0; i < nnodes; i++) {
                const int p = t.nd[i].parent;
                if (p == -1) continue;
                if (t.nd[p].c0 == -1) t.nd[p].c0 = i;
                else t.nd[p].c1 = i;
            }
        }
    }
    ThreadTrees out;
    out.nnodes = nnodes2;
    out.ntrees = 0;
    out.start_coord = a.start_coord;
    auto push = [&](const Tree &t, const int *spr, int blocklen, const std::vector<int> *mp) {
        for (int i = 0; i < nnodes2; i++) {
            out.ptrees.push_back(t.nd[i].parent);
            out.ages.push_back(t.nd[i].age);
            out.c0.push_back(t.nd[i].c0);
            out.c1.push_back(t.nd[i].c1);
            out.mapping.push_back(mp ? (*mp)[i] : -1);
        }
        for (int k = 0; k < 4; k++) out.sprs.push_back(spr[k]);
        out.blocklens.push_back(blocklen);
        out.ntrees++;
    };
    int irec = 0, end = 0;
    Tree last_tree;
    int last_node = -1;
    for (int b = 0; b < B; b++) {
        Tree tree = in[b];
        int start = end;
        end += a.blocklens[b];
        int sn, st;
        if (!state_of(in[b], nnodes, T, path[start], sn, st)) {
            err = "add_arg_thread: a path entry is not a state of its tree";
            return false;
        }
        add_tree_branch(tree, nnodes, sn, st);
        int spr[4] = {-1, -1, -1, -1};
        std::vector<int> mapping;
        const bool has_map = b > 0;
        if (has_map) {
            for (int k = 0; k < 4; k++) spr[k] = a.sprs[(size_t)b * 4 + k];
            mapping.assign(nnodes2, -1);
            if (!a.mapping.empty()) {
                for (int i = 0; i < nnodes; i++) mapping[i] = a.mapping[(size_t)b * nnodes + i];
            } else {  // make_node_mapping (local_tree.h:767-776)
                for (int i = 0; i < nnodes; i++) mapping[i] = i;
                mapping[a.ptrees[(size_t)(b - 1) * nnodes + spr[0]]] = -1;
            }
            if (!add_spr_branch(tree, last_tree, sn, st, last_node, spr, mapping, newleaf,
                                displaced, newcoal, nnodes2)) {
                err = "add_arg_thread: inconsistent SPR between neighbouring trees";
                return false;
            }
        }
        // split the block at each of its recombinations
        Tree cur = tree;
        int cur_spr[4] = {spr[0], spr[1], spr[2], spr[3]};
        std::vector<int> cur_map = mapping;
        bool cur_has_map = has_map;
        for (; irec < nrec && rec_pos[irec] < end; irec++) {
            const int pos = rec_pos[irec];
            int stn, stt, ltn, ltt;
            if (!state_of(in[b], nnodes, T, path[pos], stn, stt) ||
                !state_of(in[b], nnodes, T, path[pos - 1], ltn, ltt)) {
                err = "add_arg_thread: a path entry is not a state of its tree";
                return false;
            }
            int spr2[4];
            spr2[0] = rec_node[irec];
            spr2[1] = rec_time[irec];
            if (spr2[0] == newleaf) spr2[0] = displaced;
            if (spr2[0] == -1) {  // recombination on the new branch, coalescence as the thread
                spr2[0] = newleaf;
                spr2[2] = stn;
                if (spr2[2] == newleaf) spr2[2] = displaced;
                if (stn == ltn && stt > ltt) spr2[2] = newcoal;
            } else {  // recombination in the ARG, coalescence on the new branch
                if (spr2[0] < 0 || spr2[0] >= nnodes2) {
                    err = "add_arg_thread: a recombination node out of range";
                    return false;
                }
                spr2[2] = stt > ltt ? cur.nd[newleaf].parent : newleaf;
            }
            spr2[3] = stt;
            if (cur.nd[spr2[0]].parent < 0) {
                err = "add_arg_thread: a recombination on the root";
                return false;
            }
            std::vector<int> map2(nnodes2);
            for (int j = 0; j < nnodes2; j++) map2[j] = j;
            map2[cur.nd[spr2[0]].parent] = -1;
            Tree nt = cur;
            apply_spr(nt, spr2);
            const int block_end = irec < nrec - 1 ? std::min(rec_pos[irec + 1], end) : end;
            push(cur, cur_spr, pos - start, cur_has_map ? &cur_map : nullptr);
            cur = nt;
            for (int k = 0; k < 4; k++) cur_spr[k] = spr2[k];
            cur_map = map2;
            cur_has_map = true;
            start = pos;
            (void)block_end;
        }
        push(cur, cur_spr, end - start, cur_has_map ? &cur_map : nullptr);
        last_tree = cur;
        int ln, lt;
        if (!state_of(in[b], nnodes, T, path[end - 1], ln, lt)) {
            err = "add_arg_thread: a path entry is not a state of its tree";
            return false;
        }
        last_node = ln == newleaf ? displaced : ln;
    }
    if (irec != nrec) {
        err = "add_arg_thread: a recombination outside the trees";
        return false;
    }
    a = std::move(out);
    return true;
}

}  // namespace awg

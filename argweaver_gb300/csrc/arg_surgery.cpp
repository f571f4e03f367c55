// ARG surgery on the host. Adding a sampled thread (add_arg_thread, thread.cpp:272-422):
// the new leaf joins every local tree at the state its thread takes at the tree's first
// column, each sampled recombination splits its tree in two by an SPR, and the node
// mappings and SPRs between neighbouring trees are renamed for the two new nodes
// (add_spr_branch, thread.cpp:176-269). Removing a leaf's thread (remove_arg_thread,
// thread.cpp:425-556): the inverse, with trees whose SPR disappears merged into their
// neighbour. Pointer surgery on a few hundred nodes per tree: host work between the
// device's threading passes.
//
// Node names follow the reference: the new leaf takes the name nleaves, the node that had
// it moves to nnodes (moved_id), the new coalescence node is nnodes + 1. Child order is
// kept as the reference keeps it (it decides which child a later SPR replaces), so the
// handle stores children next to parents.

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "arg_surgery.h"

namespace awg {

namespace {

struct Node {
    int parent = -1, c0 = -1, c1 = -1, age = 0;
};

struct Tree {
    std::vector<Node> nd;
    int root = -1;
};

struct Spr4 {
    int v[4];
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
    const int leaf_id = nleaves, moved_id = nnodes, join_id = nnodes + 1;
    t.nd.resize(nnodes + 2);
    const int target = node != leaf_id ? node : moved_id;
    const int parent = t.nd[node].parent;
    const int target_up = parent != leaf_id ? parent : moved_id;
    if (leaf_id < moved_id) rename_node(t, leaf_id, moved_id);
    t.nd[leaf_id] = Node{join_id, -1, -1, 0};
    t.nd[join_id] = Node{target_up, leaf_id, target, time};
    t.nd[target].parent = join_id;
    if (target_up != -1) {
        if (t.nd[target_up].c0 == target) t.nd[target_up].c0 = join_id;
        else t.nd[target_up].c1 = join_id;
    }
    if (t.nd[join_id].parent == -1) t.root = join_id;
    else t.root = t.root != leaf_id ? t.root : moved_id;
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
                    int last_node, int *spr, std::vector<int> &mapping, int leaf_id,
                    int moved_id, int join_id, int nnodes2) {
    const int last_target = last_node != leaf_id ? last_node : moved_id;
    const int target = state_node != leaf_id ? state_node : moved_id;
    mapping[moved_id] = mapping[leaf_id];
    mapping[leaf_id] = leaf_id;
    mapping[join_id] = join_id;
    for (int i = leaf_id + 1; i < nnodes2; i++)
        if (mapping[i] == leaf_id) mapping[i] = moved_id;
    if (spr[0] == leaf_id) spr[0] = moved_id;
    if (spr[2] == leaf_id) spr[2] = moved_id;
    if (mapping[spr[0]] < 0) return false;
    const int recoal = t.nd[mapping[spr[0]]].parent;
    if (recoal == join_id) {
        if (mapping[last_target] == target) {
            spr[0] = join_id;  // recombination above the coalescence state: renamed
        } else {
            const int sn = state_node != leaf_id ? state_node : moved_id;
            if (sn == mapping[spr[0]]) {  // mediated coalescence
                spr[2] = leaf_id;
                spr[3] = state_time;
            }  // else the new branch escapes: nothing to rename
        }
    } else if (recoal != -1 && (t.nd[recoal].c0 == join_id || t.nd[recoal].c1 == join_id)) {
        if (last.nd[spr[2]].parent == join_id) spr[2] = join_id;
    }
    if (last.nd[spr[0]].parent == join_id) {  // join_id was the broken node
        mapping[join_id] = -1;
        const int p = last.nd[join_id].parent;
        if (p != -1) mapping[p] = join_id;
    } else {  // follow a child without the recombination or coalescence down to a mapped node
        int x = join_id;
        for (int steps = 0;; steps++) {
            if (steps > nnodes2) return false;
            int y = last.nd[x].c0;
            if (y == spr[2] || y == spr[0]) y = last.nd[x].c1;
            x = y;
            if (x < 0) return false;
            if (mapping[x] != -1) break;
        }
        mapping[join_id] = t.nd[mapping[x]].parent;
    }
    return true;
}

}  // namespace

bool add_arg_thread(ThreadTrees &a, int T, const int *path, int seqlen, const int *rec_pos,
                    const int *rec_node, const int *rec_time, int nrec, std::string &err) {
    const int nnodes = a.nnodes, nnodes2 = nnodes + 2, B = a.ntrees;
    const int nleaves = (nnodes + 1) / 2;
    const int leaf_id = nleaves, moved_id = nnodes, join_id = nnodes + 1;
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
            if (!add_spr_branch(tree, last_tree, sn, st, last_node, spr, mapping, leaf_id,
                                moved_id, join_id, nnodes2)) {
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
            if (spr2[0] == leaf_id) spr2[0] = moved_id;
            if (spr2[0] == -1) {  // recombination on the new branch, coalescence as the thread
                spr2[0] = leaf_id;
                spr2[2] = stn;
                if (spr2[2] == leaf_id) spr2[2] = moved_id;
                if (stn == ltn && stt > ltt) spr2[2] = join_id;
            } else {  // recombination in the ARG, coalescence on the new branch
                if (spr2[0] < 0 || spr2[0] >= nnodes2) {
                    err = "add_arg_thread: a recombination node out of range";
                    return false;
                }
                spr2[2] = stt > ltt ? cur.nd[leaf_id].parent : leaf_id;
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
        last_node = ln == leaf_id ? moved_id : ln;
    }
    if (irec != nrec) {
        err = "add_arg_thread: a recombination outside the trees";
        return false;
    }
    a = std::move(out);
    return true;
}

namespace {

// remove_tree_branch (thread.cpp:102-163): the leaf and its coalescence node leave the
// tree; the last leaf and the nodes nnodes-2, nnodes-1 move into the holes (displace[]:
// every old name's new one, -1 for the two removed)
void remove_tree_branch(Tree &t, int nnodes, int remove_leaf, std::vector<int> &displace) {
    const int last_leaf = (nnodes + 1) / 2 - 1;
    const int remove_coal = t.nd[remove_leaf].parent;
    const int coal_child =
        t.nd[remove_coal].c0 == remove_leaf ? t.nd[remove_coal].c1 : t.nd[remove_coal].c0;
    const int coal_parent = t.nd[remove_coal].parent;
    t.nd[coal_child].parent = coal_parent;
    if (coal_parent != -1) {
        if (t.nd[coal_parent].c0 == remove_coal) t.nd[coal_parent].c0 = coal_child;
        else t.nd[coal_parent].c1 = coal_child;
    }
    displace.assign(nnodes, 0);
    for (int i = 0; i < nnodes; i++) displace[i] = i;
    displace[remove_leaf] = -1;
    displace[remove_coal] = -1;
    if (last_leaf != remove_leaf) {
        displace[last_leaf] = remove_leaf;
        rename_node(t, last_leaf, remove_leaf);
    }
    int hole = last_leaf;
    if (remove_coal != nnodes - 2) {
        displace[nnodes - 2] = hole;
        rename_node(t, nnodes - 2, hole);
        hole = remove_coal;
    }
    if (remove_coal != nnodes - 1) {
        displace[nnodes - 1] = hole;
        rename_node(t, nnodes - 1, hole);
    }
    int root = t.root;
    if (root == remove_coal) root = coal_child;
    if (root == nnodes - 2) root = last_leaf;
    if (root == nnodes - 1) root = hole;
    t.root = root;
    t.nd.resize(nnodes - 2);
}

}  // namespace

namespace {

// The trees of a handle with their children (stored order, else index order), SPRs (the
// first tree's null) and mappings from the previous tree (make_node_mapping,
// local_tree.h:767-776, where none are stored).
bool load_trees(const ThreadTrees &a, std::vector<Tree> &trees,
                std::vector<std::vector<int>> &maps, std::vector<Spr4> &sprs, const char *who,
                std::string &err) {
    const int nnodes = a.nnodes, B = a.ntrees;
    trees.assign(B, Tree());
    maps.assign(B, std::vector<int>());
    sprs.assign(B, Spr4{{-1, -1, -1, -1}});
    for (int b = 0; b < B; b++) {
        Tree &t = trees[b];
        t.nd.resize(nnodes);
        for (int i = 0; i < nnodes; i++) {
            t.nd[i].parent = a.ptrees[(size_t)b * nnodes + i];
            t.nd[i].age = a.ages[(size_t)b * nnodes + i];
            if (t.nd[i].parent < -1 || t.nd[i].parent >= nnodes) {
                err = std::string(who) + ": a parent out of range";
                return false;
            }
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
        if (b == 0) continue;
        for (int k = 0; k < 4; k++) sprs[b].v[k] = a.sprs[(size_t)b * 4 + k];
        const int r = sprs[b].v[0], c = sprs[b].v[2];
        if (r < 0 || r >= nnodes || c < 0 || c >= nnodes) {
            err = std::string(who) + ": an SPR node out of range";
            return false;
        }
        if (!a.mapping.empty()) {
            maps[b].assign(a.mapping.begin() + (size_t)b * nnodes,
                           a.mapping.begin() + (size_t)(b + 1) * nnodes);
        } else {
            maps[b].resize(nnodes);
            for (int i = 0; i < nnodes; i++) maps[b][i] = i;
            const int broken = trees[b - 1].nd[r].parent;
            if (broken >= 0) maps[b][broken] = -1;
        }
    }
    return true;
}

// remove_null_sprs (local_tree.cpp:409-469): a tree whose successor has no SPR is absorbed
// by it (block lengths add, the mappings compose, its SPR moves over; the first tree's
// successor becomes the first tree). The first n nodes of each tree are kept.
ThreadTrees merge_null_sprs(const std::vector<Tree> &trees, std::vector<std::vector<int>> &maps,
                            const std::vector<Spr4> &sprs, const std::vector<int> &blocklens,
                            int n, int start_coord, const std::vector<int> &seqids) {
    ThreadTrees out;
    out.nnodes = n;
    out.start_coord = start_coord;
    out.seqids = seqids;
    struct Pending {
        int b, blocklen;
        Spr4 spr;
        std::vector<int> map;
        bool has_map;
    };
    auto emit = [&](const Pending &p) {
        const Tree &t = trees[p.b];
        for (int i = 0; i < n; i++) {
            out.ptrees.push_back(t.nd[i].parent);
            out.ages.push_back(t.nd[i].age);
            out.c0.push_back(t.nd[i].c0);
            out.c1.push_back(t.nd[i].c1);
            out.mapping.push_back(p.has_map ? p.map[i] : -1);
        }
        for (int k = 0; k < 4; k++) out.sprs.push_back(p.spr.v[k]);
        out.blocklens.push_back(p.blocklen);
        out.ntrees++;
    };
    const int B = (int)trees.size();
    Pending cur{0, blocklens[0], sprs[0], {}, false};
    for (int b = 1; b < B; b++) {
        Pending nx{b, blocklens[b], sprs[b], std::move(maps[b]), true};
        nx.map.resize(n);
        if (nx.spr.v[0] == -1) {  // no SPR into tree b: tree cur merges into it
            if (!cur.has_map) {
                nx.has_map = false;
            } else {
                std::vector<int> comp(n);
                for (int i = 0; i < n; i++) comp[i] = cur.map[i] != -1 ? nx.map[cur.map[i]] : -1;
                nx.map = std::move(comp);
                nx.spr = cur.spr;
            }
            nx.blocklen += cur.blocklen;
        } else {
            emit(cur);
        }
        cur = std::move(nx);
    }
    emit(cur);
    return out;
}

}  // namespace

bool remove_arg_thread(ThreadTrees &a, int seqid, std::string &err) {
    const int nnodes = a.nnodes, B = a.ntrees;
    const int nleaves = (nnodes + 1) / 2, last_leaf = nleaves - 1;
    std::vector<int> seqids = a.seqids;
    if (seqids.empty())
        for (int i = 0; i < nleaves; i++) seqids.push_back(i);
    if ((int)seqids.size() != nleaves || nnodes != 2 * nleaves - 1) {
        err = "remove_arg_thread: the sequence ids do not match the leaves";
        return false;
    }
    int remove_leaf = -1;
    for (int i = 0; i < (int)seqids.size(); i++)
        if (seqids[i] == seqid) {
            remove_leaf = i;
            break;
        }
    if (remove_leaf < 0) {
        err = "remove_arg_thread: no leaf holds that sequence";
        return false;
    }
    long long total = 0;
    for (int b = 0; b < B; b++) total += a.blocklens[b];
    if (nnodes == 3) {  // the trunk genealogy is left (make_trunk, local_tree.h:576-590)
        const int other = seqids[1 - remove_leaf];
        ThreadTrees out;
        out.ntrees = 1;
        out.nnodes = 1;
        out.start_coord = a.start_coord;
        out.ptrees = {-1};
        out.ages = {0};
        out.sprs = {-1, -1, -1, -1};
        out.blocklens = {(int)total};
        out.c0 = {-1};
        out.c1 = {-1};
        out.seqids = {other};
        a = std::move(out);
        return true;
    }
    if (nnodes < 3) {
        err = "remove_arg_thread: no thread to remove";
        return false;
    }
    std::vector<Tree> trees;
    std::vector<std::vector<int>> maps;
    std::vector<Spr4> sprs;
    if (!load_trees(a, trees, maps, sprs, "remove_arg_thread", err)) return false;
    std::vector<int> displace;
    for (int b = 0; b < B; b++) {
        Tree &t = trees[b];
        const int remove_coal = t.nd[remove_leaf].parent;
        if (remove_coal < 0) {
            err = "remove_arg_thread: the leaf has no parent";
            return false;
        }
        const int coal_time = t.nd[remove_coal].age;
        int coal_child =
            t.nd[remove_coal].c0 == remove_leaf ? t.nd[remove_coal].c1 : t.nd[remove_coal].c0;
        remove_tree_branch(t, nnodes, remove_leaf, displace);
        if (b > 0) {  // this mapping's targets renamed
            std::vector<int> &m = maps[b];
            for (int i = 0; i < nnodes - 2; i++) m[i] = m[i] != -1 ? displace[m[i]] : -1;
        }
        if (b + 1 == B) continue;
        // the next mapping's sources renamed (the moved nodes keep their targets)
        std::vector<int> &m = maps[b + 1];
        if (displace[last_leaf] != -1) m[displace[last_leaf]] = m[last_leaf];
        if (displace[nnodes - 2] != -1) m[displace[nnodes - 2]] = m[nnodes - 2];
        if (displace[nnodes - 1] != -1) m[displace[nnodes - 1]] = m[nnodes - 1];
        int *spr = sprs[b + 1].v;
        coal_child = displace[coal_child];
        auto set_null = [&]() { spr[0] = spr[1] = spr[2] = spr[3] = -1; };
        if (spr[0] < 0 || spr[0] >= nnodes || spr[2] < 0 || spr[2] >= nnodes) {
            err = "remove_arg_thread: an SPR node out of range";
            return false;
        }
        if (spr[0] == remove_leaf) { set_null(); continue; }  // recombination on the branch
        spr[0] = spr[0] == remove_coal ? coal_child : displace[spr[0]];
        if (spr[0] == coal_child && t.nd[coal_child].parent == -1) { set_null(); continue; }
        if (spr[2] == remove_leaf) {  // mediated coalescence
            spr[2] = coal_child;
            spr[3] = coal_time;
        } else if (spr[2] == remove_coal) {
            spr[2] = coal_child;
        } else {
            spr[2] = displace[spr[2]];
        }
        if (spr[0] == spr[2]) { set_null(); continue; }  // a bubble
    }
    seqids[remove_leaf] = seqids[last_leaf];
    seqids.resize(nleaves - 1);
    a = merge_null_sprs(trees, maps, sprs, a.blocklens, nnodes - 2, a.start_coord, seqids);
    return true;
}

namespace {

int sibling(const Tree &t, int v) {
    const int p = t.nd[v].parent;
    if (p == -1) return -1;
    return t.nd[p].c0 == v ? t.nd[p].c1 : t.nd[p].c0;
}

// get_recoal_node (local_tree.cpp:473-488): the first node of the next tree nothing maps to
int recoal_node(int n, const std::vector<int> &mapping) {
    std::vector<char> mapped(n, 0);
    for (int i = 0; i < n; i++)
        if (mapping[i] != -1) mapped[mapping[i]] = 1;
    for (int i = 0; i < n; i++)
        if (!mapped[i]) return i;
    return -1;
}

// get_next_removal_nodes (thread.cpp:562-591): where a removal path on `node` of tree1
// continues in the next tree: the passive branch, and the recoalescence when the SPR
// coalesces on `node`
void next_removal_nodes(const Tree &tree1, const Spr4 &spr, const std::vector<int> &mapping,
                        int node, int next[2], int recoal) {
    const int n = (int)tree1.nd.size();
    if (recoal == -1) recoal = recoal_node(n, mapping);
    next[0] = mapping[node];
    if (next[0] == -1) {  // node broken by the SPR: the sibling's branch, or the recoalescence
        const int sib = sibling(tree1, spr.v[0]);
        next[0] = spr.v[2] == sib ? recoal : mapping[sib];
    }
    next[1] = spr.v[2] == node ? recoal : -1;
}

// get_prev_removal_nodes (thread.cpp:609-647): the branches of tree1 a removal path on
// `node` of the next tree can come from
void prev_removal_nodes(const Tree &tree1, const Spr4 &spr, const std::vector<int> &mapping,
                        const std::vector<int> &inv, int node, int prev[2]) {
    prev[0] = inv[node];
    const int sib = sibling(tree1, spr.v[0]);
    if (prev[0] == -1) {  // node is the recoalescence
        prev[0] = spr.v[2];
        prev[1] = sib == spr.v[2] ? tree1.nd[sib].parent : -1;
    } else {
        prev[1] = mapping[sib] == node && sib != spr.v[2] ? tree1.nd[sib].parent : -1;
    }
}

std::vector<int> inverse_mapping(const std::vector<int> &mapping, int n) {
    std::vector<int> inv(n, -1);
    for (int i = 0; i < n; i++)
        if (mapping[i] != -1) inv[mapping[i]] = i;
    return inv;
}

// logadd and logsum (common.h:157-163,182-201)
double log_add(double a, double b) {
    if (a == -INFINITY) return b;
    if (b == -INFINITY) return a;
    return std::max(a, b) + std::log1p(std::exp(-std::fabs(a - b)));
}

double log_sum(const double *v, int n) {
    if (n == 0) return 1.0;
    double m = v[0];
    for (int i = 1; i < n; i++)
        if (v[i] > m) m = v[i];
    double e = 0.0;
    for (int i = 0; i < n; i++)
        if (v[i] - m > -15) e += std::exp(v[i] - m);
    return m + std::log(e);
}

double unit(int (*rnd)()) { return rnd() / double(RAND_MAX); }  // frand (common.h:103-104)

// one step of a removal path forward (sample_arg_removal_path_forward, thread.cpp:703-735):
// the second branch is taken when rand() < 0.5, i.e. when rand() returns 0, as there
int step_forward(const Tree &last, const Spr4 &spr, const std::vector<int> &mapping, int node,
                 int (*rnd)()) {
    int next[2];
    next_removal_nodes(last, spr, mapping, node, next, -1);
    if (next[1] == -1 || !rnd) return next[0];
    return next[int(rnd() < 0.5)];
}

}  // namespace

bool sample_removal_path(const ThreadTrees &a, int node, long long pos, int (*rnd)(), int *path,
                         std::string &err) {
    std::vector<Tree> trees;
    std::vector<std::vector<int>> maps;
    std::vector<Spr4> sprs;
    if (!load_trees(a, trees, maps, sprs, "sample_arg_removal_path", err)) return false;
    if (node < 0 || node >= a.nnodes) {
        err = "sample_arg_removal_path: node out of range";
        return false;
    }
    const int B = a.ntrees;
    int i0 = 0;
    if (pos >= 0) {  // the block holding pos (thread.cpp:772-790)
        long long end = a.start_coord;
        for (i0 = 0; i0 < B; i0++) {
            const long long start = end;
            end += a.blocklens[i0];
            if (start <= pos && pos < end) break;
        }
        if (i0 == B) {
            err = "sample_arg_removal_path: pos outside the trees";
            return false;
        }
    }
    path[i0] = node;
    for (int b = i0 + 1; b < B; b++)
        path[b] = step_forward(trees[b - 1], sprs[b], maps[b], path[b - 1], rnd);
    // backward from the block (sample_arg_removal_path_backward, thread.cpp:738-769)
    for (int b = i0 - 1; b >= 0; b--) {
        int prev[2];
        prev_removal_nodes(trees[b], sprs[b + 1], maps[b + 1],
                           inverse_mapping(maps[b + 1], a.nnodes), path[b + 1], prev);
        path[b] = prev[1] == -1 ? prev[0] : prev[int(rnd() < 0.5)];
    }
    return true;
}

// sample (common.h:272-290): the first index whose running weight reaches frand(total)
static int sample_index(const double *w, int n, int (*rnd)()) {
    double total = 0.0;
    for (int i = 0; i < n; i++) total += w[i];
    const double pick = unit(rnd) * total;
    double x = 0.0;
    for (int i = 0; i < n; i++) {
        x += w[i];
        if (x >= pick) return i;
    }
    return n - 1;
}

bool sample_removal_path_recomb(const ThreadTrees &a, double pref, int (*rnd)(), int *path,
                                std::string &err) {
    std::vector<Tree> trees;
    std::vector<std::vector<int>> maps;
    std::vector<Spr4> sprs;
    if (!load_trees(a, trees, maps, sprs, "sample_arg_removal_path_recomb", err)) return false;
    const int B = a.ntrees, n = a.nnodes;
    // forward table over branches (thread.cpp:814-878). As the reference's, the split
    // weight and the recombination preference are looked up by the later tree's node index.
    std::vector<double> fw((size_t)B * n), trans((size_t)B * n, 1.0);
    std::vector<int> back((size_t)B * n * 2, -1);
    for (int j = 0; j < n; j++) fw[j] = 1.0 / n;
    for (int b = 1; b < B; b++) {
        const std::vector<int> inv = inverse_mapping(maps[b], n);
        const int recoal = recoal_node(n, maps[b]);
        for (int j = 0; j < n; j++) {
            int next[2];
            next_removal_nodes(trees[b - 1], sprs[b], maps[b], j, next, recoal);
            trans[(size_t)(b - 1) * n + j] = next[1] != -1 ? .5 : 1.0;
            int *ptr = &back[((size_t)b * n + j) * 2];
            prev_removal_nodes(trees[b - 1], sprs[b], maps[b], inv, j, ptr);
            if (ptr[0] < 0 || ptr[0] >= n || ptr[1] >= n) {
                err = "sample_arg_removal_path_recomb: inconsistent SPR between neighbouring trees";
                return false;
            }
        }
        double norm = 0.0;
        for (int j = 0; j < n; j++) {
            const int *ptr = &back[((size_t)b * n + j) * 2];
            double sum = 0.0;
            for (int ki = 0; ki < 2; ki++)
                if (ptr[ki] != -1) sum += trans[(size_t)(b - 1) * n + j] * fw[(size_t)(b - 1) * n + ptr[ki]];
            const double emit = sprs[b].v[0] == j ? pref : 1.0 - pref;
            fw[(size_t)b * n + j] = sum * emit;
            norm += fw[(size_t)b * n + j];
        }
        for (int j = 0; j < n; j++) fw[(size_t)b * n + j] /= norm;
    }
    // the last branch, then a stochastic traceback (thread.cpp:881-903)
    int j = path[B - 1] = sample_index(&fw[(size_t)(B - 1) * n], n, rnd);
    for (int b = B - 2; b >= 0; b--) {
        const int *ptr = &back[((size_t)(b + 1) * n + j) * 2];
        if (ptr[1] == -1) {
            j = path[b] = ptr[0];
        } else {
            const double t = trans[(size_t)b * n + j];
            const double probs[2] = {fw[(size_t)b * n + ptr[0]] * t, fw[(size_t)b * n + ptr[1]] * t};
            j = path[b] = ptr[sample_index(probs, 2, rnd)];
        }
    }
    return true;
}

bool sample_removal_path_uniform(const ThreadTrees &a, int (*rnd)(), int *path, double *lntotal,
                                 std::string &err) {
    std::vector<Tree> trees;
    std::vector<std::vector<int>> maps;
    std::vector<Spr4> sprs;
    if (!load_trees(a, trees, maps, sprs, "sample_arg_removal_path_uniform", err)) return false;
    const int B = a.ntrees, n = a.nnodes;
    // log path counts and back pointers (count_arg_removal_paths, thread.cpp:914-950)
    std::vector<double> counts((size_t)B * n, 0.0);
    std::vector<int> back((size_t)B * n * 2, -1);
    for (int b = 1; b < B; b++) {
        const std::vector<int> inv = inverse_mapping(maps[b], n);
        for (int j = 0; j < n; j++) {
            int *ptr = &back[((size_t)b * n + j) * 2];
            prev_removal_nodes(trees[b - 1], sprs[b], maps[b], inv, j, ptr);
            const double *c = &counts[(size_t)(b - 1) * n];
            if (ptr[0] < 0 || ptr[0] >= n || ptr[1] >= n) {
                err = "sample_arg_removal_path_uniform: inconsistent SPR between neighbouring trees";
                return false;
            }
            counts[(size_t)b * n + j] = ptr[1] == -1 ? c[ptr[0]] : log_add(c[ptr[0]], c[ptr[1]]);
        }
    }
    // the last branch by path counts (sample, common.h:272-290), then back (thread.cpp:963-1002)
    const double *last = &counts[(size_t)(B - 1) * n];
    const double norm = log_sum(last, n);
    std::vector<double> w(n);
    double total = 0.0;
    for (int j = 0; j < n; j++) {
        w[j] = std::exp(last[j] - norm);
        total += w[j];
    }
    const double pick = unit(rnd) * total;
    double x = 0.0;
    int k = n - 1;
    for (int j = 0; j < n; j++) {
        x += w[j];
        if (x >= pick) {
            k = j;
            break;
        }
    }
    path[B - 1] = k;
    for (int b = B - 1; b > 0; b--) {
        const int *ptr = &back[((size_t)b * n + path[b]) * 2];
        if (ptr[1] == -1) {
            path[b - 1] = ptr[0];
        } else {
            const double p1 = counts[(size_t)(b - 1) * n + ptr[0]];
            const double p2 = counts[(size_t)(b - 1) * n + ptr[1]];
            path[b - 1] = std::log(unit(rnd)) < p1 - log_add(p1, p2) ? ptr[0] : ptr[1];
        }
    }
    if (lntotal) *lntotal = log_sum(last, n);
    return true;
}
namespace {

struct NodeTime {
    int node, time;
};

// The coalescence states of a tree in subtree/main-tree form, in the reference's order
// (get_coal_states_internal, states.cpp:109-155): none for a whole tree; else every main-tree
// branch from max(age, minage, subtree age) up to its parent's age, the basal branches up
// to ntimes - 2.
void internal_states(const Tree &t, int T, int minage, std::vector<NodeTime> &st) {
    st.clear();
    const int n = (int)t.nd.size();
    if (t.nd[t.root].age < T) return;
    const int sub = t.nd[t.root].c0;
    minage = std::max(minage, t.nd[sub].age);
    std::vector<char> skip(n, 0);
    skip[t.root] = 1;
    std::vector<int> stack{sub};
    while (!stack.empty()) {
        const int v = stack.back();
        stack.pop_back();
        skip[v] = 1;
        if (t.nd[v].c0 != -1) {
            stack.push_back(t.nd[v].c0);
            stack.push_back(t.nd[v].c1);
        }
    }
    for (int i = 0; i < n; i++) {
        if (skip[i]) continue;
        const int parent = t.nd[i].parent;
        const int top = parent == t.root ? T - 2 : t.nd[parent].age;
        for (int time = std::max(t.nd[i].age, minage); time <= top; time++)
            st.push_back(NodeTime{i, time});
    }
}

}  // namespace

bool remove_thread_path(ThreadTrees &a, const int *removal_path, int maxtime,
                        int *original_thread, std::string &err) {
    std::vector<Tree> trees;
    std::vector<std::vector<int>> maps;
    std::vector<Spr4> sprs;
    if (!load_trees(a, trees, maps, sprs, "remove_arg_thread_path", err)) return false;
    const int B = a.ntrees, n = a.nnodes;
    for (int b = 0; b < B; b++)
        if (removal_path[b] < 0 || removal_path[b] >= n) {
            err = "remove_arg_thread_path: a path node out of range";
            return false;
        }
    std::vector<NodeTime> orig(B, NodeTime{-1, -1});  // the removed thread, per tree
    for (int b = 0; b < B; b++) {
        Tree &t = trees[b];
        const Tree *last = b > 0 ? &trees[b - 1] : nullptr;
        const int rn = removal_path[b];
        if (rn == t.root) {  // the path has left the tree over the top: nothing to cut
            if (last && removal_path[b - 1] != last->root) maps[b][last->root] = -1;
            continue;
        }
        orig[b] = NodeTime{sibling(t, rn), t.nd[t.nd[rn].parent].age};
        // cut the branch above rn and regraft it over the root at maxtime: the tree in
        // subtree/main-tree form, the subtree the root's first child
        const int broken = t.nd[rn].parent;
        const int coal_time = t.nd[broken].age;
        const int broken_child = sibling(t, rn);
        const int cut[4] = {rn, t.nd[rn].age, t.root, maxtime};
        apply_spr(t, cut);
        const int mainr = sibling(t, rn);
        Node &root = t.nd[t.root];
        if (root.c0 == mainr) {
            root.c0 = rn;
            root.c1 = mainr;
        }
        if (last && removal_path[b - 1] != last->root) maps[b][last->root] = t.root;
        if (b + 1 == B) continue;
        // the SPR into the next tree (thread.cpp:1560-1635)
        int *spr = sprs[b + 1].v;
        std::vector<int> &m = maps[b + 1];
        auto set_null = [&]() { spr[0] = spr[1] = spr[2] = spr[3] = -1; };
        if (spr[0] == rn) { set_null(); continue; }  // recombination on the removed branch
        if (spr[0] == broken) spr[0] = broken_child;
        int next[2];
        next_removal_nodes(t, sprs[b + 1], m, rn, next, -1);
        if (spr[2] == rn) {
            if (removal_path[b + 1] == next[0]) {  // the path takes the lower branch
                if (spr[0] == broken_child) { set_null(); continue; }  // now a bubble
                spr[2] = broken_child;  // a mediated coalescence
                spr[3] = coal_time;
            }  // else the path takes the upper branch: the recoalescence stays
        } else if (spr[2] == broken) {
            spr[2] = broken_child;
        }
        if (spr[0] == spr[2]) { set_null(); continue; }  // a bubble
        const int spr_broken = t.nd[spr[0]].parent;
        if (spr_broken < 0) {
            err = "remove_arg_thread_path: a recombination on the root";
            return false;
        }
        m[spr_broken] = -1;
    }
    if (original_thread) {  // the removed thread as states of the cut trees (thread.cpp:1638-1665)
        std::vector<NodeTime> states;
        std::vector<int> nodes(n);
        int col = 0;
        for (int b = 0; b < B; b++) {
            // get_actual_nodes (thread.cpp:1452-1477): names in the last tree the merge keeps;
            // the mapping test reads mapping[i], as the reference's does
            for (int i = 0; i < n; i++) nodes[i] = i;
            int b2 = b + 1;
            for (; b2 < B && sprs[b2].v[0] == -1; b2++)
                for (int i = 0; i < n; i++)
                    nodes[i] = maps[b2][i] != -1 && nodes[i] != -1 ? maps[b2][nodes[i]] : -1;
            internal_states(trees[b2 - 1], maxtime - 1, 0, states);
            int k = 0;
            if (!states.empty()) {
                const NodeTime o = orig[b];
                const int node = o.node >= 0 ? nodes[o.node] : -1;
                k = -1;
                for (int j = 0; j < (int)states.size() && k < 0; j++)
                    if (states[j].node == node && states[j].time == o.time) k = j;
                if (k < 0) {
                    err = "remove_arg_thread_path: the removed thread is no state of its tree";
                    return false;
                }
            }
            for (int c = 0; c < a.blocklens[b]; c++) original_thread[col++] = k;
        }
    }
    a = merge_null_sprs(trees, maps, sprs, a.blocklens, n, a.start_coord, a.seqids);
    return true;
}

namespace {

// add_spr_branch for an internal branch (thread.cpp:1204-1311): the SPR into `t` and its
// mapping renamed for the regrafted subtree's new coalescence node
bool add_spr_branch_internal(const Tree &t, const Tree &last, NodeTime state, NodeTime last_state,
                             int *spr, std::vector<int> &mapping, int sub, int last_sub) {
    const int n = (int)t.nd.size();
    auto ok = [n](int v) { return v >= 0 && v < n; };
    const int last_newcoal = last.nd[last_sub].parent;
    int join_id;
    if (state.node != -1) {
        join_id = t.nd[sub].parent;
    } else if (mapping[last_sub] != -1) {  // a whole tree
        join_id = t.nd[mapping[last_sub]].parent;
    } else {
        const int sib = sibling(last, spr[0]);
        if (!ok(sib) || !ok(mapping[sib])) return false;
        join_id = t.nd[mapping[sib]].parent;
    }
    if (!ok(last_newcoal) || !ok(mapping[spr[0]])) return false;
    mapping[last_newcoal] = join_id;
    const int recoal = t.nd[mapping[spr[0]]].parent;
    if (recoal == join_id) {
        if (mapping[last_state.node] == state.node) {
            spr[0] = last_newcoal;  // the recombination is above the coalescence: renamed
        } else if (spr[3] == last.nd[last_newcoal].age && state.node == mapping[spr[0]]) {
            // a mediated coalescence
            spr[2] = state.time < last.nd[last_sub].age ? sibling(last, spr[0]) : last_sub;
            spr[3] = state.time;
        }  // else the new branch escapes: nothing to rename
    } else if (recoal != -1 && (t.nd[recoal].c0 == join_id || t.nd[recoal].c1 == join_id)) {
        if (last.nd[spr[2]].parent == last_newcoal) spr[2] = last_newcoal;
    }
    if (last.nd[spr[0]].parent == last_newcoal) {  // last_newcoal was the broken node
        mapping[last_newcoal] = -1;
        const int p = last.nd[last_newcoal].parent;
        if (p != -1) mapping[p] = join_id;
    } else {  // a child of last_newcoal without the recombination or coalescence on it
        const int x = last_newcoal;
        int y = last.nd[x].c0;
        if (y == spr[2]) y = last.nd[x].c1;
        if (!ok(y)) return false;
        if (mapping[y] == -1) y = sibling(last, spr[0]);
        if (y == spr[2]) y = last.nd[x].c1;
        if (!ok(y) || !ok(mapping[y])) return false;
        mapping[last_newcoal] = t.nd[mapping[y]].parent;
    }
    return last.nd[spr[0]].parent != -1;
}

}  // namespace

bool add_thread_path(ThreadTrees &a, int T, int minage, const int *path, int seqlen,
                     const int *rec_pos, const int *rec_node, const int *rec_time, int nrec,
                     std::string &err) {
    std::vector<Tree> in;
    std::vector<std::vector<int>> maps;
    std::vector<Spr4> sprs;
    if (!load_trees(a, in, maps, sprs, "add_arg_thread_path", err)) return false;
    const int n = a.nnodes, B = a.ntrees;
    long long total = 0;
    for (int b = 0; b < B; b++) total += a.blocklens[b];
    if (total != seqlen) {
        err = "add_arg_thread_path: the path does not cover the trees";
        return false;
    }
    for (int r = 0; r < nrec; r++)
        if (rec_pos[r] <= 0 || rec_pos[r] >= seqlen || (r > 0 && rec_pos[r] <= rec_pos[r - 1])) {
            err = "add_arg_thread_path: recombination columns must increase within the region";
            return false;
        }
    ThreadTrees out;
    out.nnodes = n;
    out.start_coord = a.start_coord;
    out.seqids = a.seqids;
    auto push = [&](const Tree &t, const int *spr, int blocklen, const std::vector<int> *mp) {
        for (int i = 0; i < n; i++) {
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
    std::vector<NodeTime> states;
    auto state_at = [&](int col, NodeTime &s) {
        const int k = path[col];
        if (k < 0 || k >= (int)states.size()) return false;
        s = states[k];
        return true;
    };
    Tree last_tree;
    NodeTime last_state{0, 0};  // State() (states.h): node 0 until the first tree is seen
    int last_sub = -1, irec = 0, end = 0;
    for (int b = 0; b < B; b++) {
        Tree tree = in[b];
        int start = end;
        end += a.blocklens[b];
        const int sub = tree.nd[tree.root].c0;
        internal_states(in[b], T, minage, states);
        NodeTime state{-1, -1};
        if (tree.nd[tree.root].age > T) {  // a partial tree: regraft the subtree at the state
            if (sub < 0 || !state_at(start, state)) {
                err = "add_arg_thread_path: a path entry is not a state of its tree";
                return false;
            }
            const int graft[4] = {sub, tree.nd[sub].age, state.node, state.time};
            apply_spr(tree, graft);
        }
        int spr[4] = {sprs[b].v[0], sprs[b].v[1], sprs[b].v[2], sprs[b].v[3]};
        std::vector<int> mapping = maps[b];
        const bool has_map = b > 0;
        if (has_map && last_state.node != -1 &&
            !add_spr_branch_internal(tree, last_tree, state, last_state, spr, mapping, sub,
                                     last_sub)) {
            err = "add_arg_thread_path: inconsistent SPR between neighbouring trees";
            return false;
        }
        // split the block at each of its recombinations
        Tree cur = tree;
        int cur_spr[4] = {spr[0], spr[1], spr[2], spr[3]};
        std::vector<int> cur_map = mapping;
        bool cur_has_map = has_map;
        for (; irec < nrec && rec_pos[irec] < end; irec++) {
            const int pos = rec_pos[irec];
            if (!state_at(pos, state) || !state_at(pos - 1, last_state)) {
                err = "add_arg_thread_path: a path entry is not a state of its tree";
                return false;
            }
            const int join_id = cur.nd[sub].parent;
            int spr2[4] = {rec_node[irec], rec_time[irec], -1, state.time};
            if (spr2[0] < 0 || spr2[0] >= n) {
                err = "add_arg_thread_path: a recombination node out of range";
                return false;
            }
            if (spr2[0] == sub) {  // on the regrafted branch: coalescence as the thread
                spr2[2] = state.node == last_state.node && state.time > last_state.time
                              ? join_id : state.node;
            } else {  // in the main tree: coalescence on the regrafted branch
                spr2[2] = state.time > last_state.time ? cur.nd[sub].parent : sub;
            }
            const int broken = cur.nd[spr2[0]].parent;
            if (broken < 0) {
                err = "add_arg_thread_path: a recombination on the root";
                return false;
            }
            std::vector<int> map2(n);
            for (int j = 0; j < n; j++) map2[j] = j;
            map2[broken] = -1;
            Tree nt = cur;
            apply_spr(nt, spr2);
            push(cur, cur_spr, pos - start, cur_has_map ? &cur_map : nullptr);
            cur = std::move(nt);
            for (int k = 0; k < 4; k++) cur_spr[k] = spr2[k];
            cur_map = std::move(map2);
            cur_has_map = true;
            start = pos;
        }
        push(cur, cur_spr, end - start, cur_has_map ? &cur_map : nullptr);
        last_tree = std::move(cur);
        last_state = state;
        last_sub = sub;
    }
    if (irec != nrec) {
        err = "add_arg_thread_path: a recombination outside the trees";
        return false;
    }
    a = std::move(out);
    return true;
}

bool thread_times(const ThreadTrees &a, int T, const int *path, int *path_times,
                  std::string &err) {
    std::vector<Tree> trees;
    std::vector<std::vector<int>> maps;
    std::vector<Spr4> sprs;
    if (!load_trees(a, trees, maps, sprs, "arghmm_get_thread_times", err)) return false;
    std::vector<NodeTime> states;
    long long end = a.start_coord;
    for (int b = 0; b < a.ntrees; b++) {
        const long long start = end;
        end += a.blocklens[b];
        internal_states(trees[b], T, 0, states);
        for (long long i = start; i < end; i++) {
            if (states.empty()) {  // a whole tree: no thread here (the reference reads past)
                path_times[i] = -1;
                continue;
            }
            if (path[i] < 0 || path[i] >= (int)states.size()) {
                err = "arghmm_get_thread_times: a path entry is not a state of its tree";
                return false;
            }
            path_times[i] = states[path[i]].time;
        }
    }
    return true;
}

}  // namespace awg

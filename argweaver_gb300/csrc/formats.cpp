// The input formats arg-sample reads ahead of the threading HMM, on the host: sites files
// (sequences.cpp:133-297), site compression (find_compress_cols / compress_sites /
// make_sequences_from_sites, sequences.cpp:315-343,523-623), SMC local trees
// (read_local_trees / parse_local_tree, local_tree.cpp:1022-1560) and their compression
// (compress_local_trees, local_tree.cpp:818-850; SitesMapping::compress_blocks,
// sequences.h:300-322), as arg-sample chains them (arg-sample.cpp:996-1155). Files ending
// in ".gz" go through `gzip -dc` / `gzip -c` (compress.cpp:12-45). Writers produce files the
// reference reads back.

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "argweaver_gb300.h"
#include "formats.h"

struct awg_arg_input {
    std::vector<std::string> names;  // sequence names, sites order
    std::string chrom;
    int seqlen = 0, start_coord = 0;
    std::vector<char> seqs;  // [nseqs][seqlen] compressed sequences
    // local trees (empty without an SMC file), leaves permuted so leaf i is sequence i
    int ntrees = 0, nnodes = 0;
    std::vector<int> ptrees, ages, sprs, blocklens;
};

namespace {

thread_local std::string f_err;

void fail(const std::string &msg) {
    f_err = msg;
    fprintf(stderr, "argweaver_gb300: %s\n", msg.c_str());
}

std::string quote(const std::string &s) {
    std::string q = "'";
    for (char c : s) {
        if (c == '\'') q += "'\\''";
        else q += c;
    }
    return q + "'";
}

bool gz_name(const char *path) {
    const size_t n = strlen(path);
    return n > 3 && strcmp(path + n - 3, ".gz") == 0;
}

// a stream over a plain or gzip-compressed file
struct Stream {
    FILE *f = nullptr;
    bool pipe = false;
    Stream(const char *path, bool write) {
        if (gz_name(path)) {
            pipe = true;
            const std::string cmd = write ? "gzip -c > " + quote(path) : "gzip -dc < " + quote(path);
            if (!write) {
                FILE *probe = fopen(path, "rb");
                if (!probe) return;
                fclose(probe);
            }
            f = popen(cmd.c_str(), write ? "w" : "r");
        } else {
            f = fopen(path, write ? "w" : "r");
        }
    }
    ~Stream() { close(); }
    int close() {
        int rc = 0;
        if (f) rc = pipe ? pclose(f) : fclose(f);
        f = nullptr;
        return rc;
    }
};

bool get_line(FILE *f, std::string &line) {
    line.clear();
    int c;
    bool any = false;
    while ((c = fgetc(f)) != EOF) {
        any = true;
        if (c == '\n') break;
        line += (char)c;
    }
    while (!line.empty() && (line.back() == '\r' || line.back() == '\n')) line.pop_back();
    return any;
}

std::vector<std::string> split_tabs(const std::string &s) {
    std::vector<std::string> out;
    size_t a = 0;
    while (true) {
        const size_t b = s.find('\t', a);
        out.push_back(s.substr(a, b == std::string::npos ? std::string::npos : b - a));
        if (b == std::string::npos) break;
        a = b + 1;
    }
    return out;
}

int base_code(char c) {
    switch (c) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    default: return -1;
    }
}

// ------------------------------------------------------------------------- sites

struct Sites {
    std::vector<std::string> names;
    std::string chrom;
    int start_coord = 0, end_coord = 0;
    std::vector<int> positions;
    std::vector<std::string> cols;
};

// read_sites (sequences.cpp:172-297), with its conventions: REGION is 1-based inclusive and
// becomes [start - 1, end); a site line is kept when its 1-based position lies in
// [start_coord, end_coord) as read (before the conversion), bases are upper-cased and must
// be ACGT or N, positions strictly increasing.
bool read_sites(FILE *f, Sites &s, int sub_start, int sub_end) {
    std::string line;
    int nseqs = 0, lineno = 0;
    while (get_line(f, line)) {
        lineno++;
        if (line.compare(0, 6, "NAMES\t") == 0) {
            s.names = split_tabs(line.substr(6));
            nseqs = (int)s.names.size();
            for (int i = 0; i < nseqs; i++)
                if (s.names[i].empty()) {
                    fail("sites: zero-length sequence name (line " + std::to_string(lineno) + ")");
                    return false;
                }
        } else if (line.compare(0, 7, "REGION\t") == 0) {
            char chrom[51];
            if (sscanf(line.c_str(), "REGION\t%50s\t%d\t%d", chrom, &s.start_coord, &s.end_coord) != 3) {
                fail("sites: bad REGION line");
                return false;
            }
            s.chrom = chrom;
            s.start_coord--;
            if (sub_start != -1) s.start_coord = sub_start;
            if (sub_end != -1) s.end_coord = sub_end;
        } else if (line.compare(0, 6, "RANGE\t") == 0) {
            fail("sites: deprecated RANGE line (use REGION)");
            return false;
        } else {
            int position;
            if (sscanf(line.c_str(), "%d\t", &position) != 1) {
                fail("sites: first column is not an integer (line " + std::to_string(lineno) + ")");
                return false;
            }
            if (position < s.start_coord || position >= s.end_coord) continue;
            const size_t tab = line.find('\t');
            std::string col = tab == std::string::npos ? std::string() : line.substr(tab + 1);
            if ((int)col.size() != nseqs) {
                fail("sites: the number of bases does not match the number of sequences (line " +
                     std::to_string(lineno) + ")");
                return false;
            }
            for (char &c : col) {
                c = (char)toupper((unsigned char)c);
                if (c != 'N' && base_code(c) < 0) {
                    fail("sites: invalid sequence characters (line " + std::to_string(lineno) + ")");
                    return false;
                }
            }
            position--;
            if (!s.positions.empty() && s.positions.back() >= position) {
                fail("sites: positions must be sorted and unique (line " + std::to_string(lineno) + ")");
                return false;
            }
            s.positions.push_back(position);
            s.cols.push_back(col);
        }
    }
    return true;
}

struct SitesMapping {
    int src_start = 0, src_end = 0, dst_start = 0, dst_end = 0;
    std::vector<int> src_pos, dst_col, kept_pos;
};

// find_compress_cols (sequences.cpp:523-592): every variant column is kept; the others
// are represented by one column per `compress` bases
bool find_compress_cols(const Sites &s, int compress, SitesMapping &m) {
    const int ncols = (int)s.positions.size();
    m.src_start = s.start_coord;
    m.src_end = s.end_coord;
    if (compress == 1) {
        for (int i = s.start_coord; i < s.end_coord; i++) m.kept_pos.push_back(i);
        for (int i = 0; i < ncols; i++) {
            m.src_pos.push_back(s.positions[i]);
            m.dst_col.push_back(s.positions[i] - s.start_coord);
        }
        m.dst_start = 0;
        m.dst_end = s.end_coord - s.start_coord;
        return true;
    }
    int ncol = 0, block_end = s.start_coord + compress;
    const int half = compress / 2;
    for (int i = 0; i < ncols; i++) {
        const int col = s.positions[i];
        while (col >= block_end) {
            m.kept_pos.push_back(block_end - half);
            block_end += compress;
            ncol++;
        }
        m.src_pos.push_back(col);
        m.dst_col.push_back(ncol);
        m.kept_pos.push_back(col);
        block_end += compress;
        ncol++;
        if (block_end - compress > s.end_coord && i != ncols - 1) return false;
    }
    while (s.end_coord >= block_end) {
        m.kept_pos.push_back(block_end - half);
        block_end += compress;
        ncol++;
    }
    m.dst_start = 0;
    const int dst_end = (s.end_coord - s.start_coord) / compress;
    m.dst_end = ncols > 0 ? std::max(m.dst_col[ncols - 1] + 1, dst_end) : dst_end;
    return true;
}

// compress_sites + make_sequences_from_sites (sequences.cpp:315-343,598-606): variant
// columns at their compressed positions, every other column the default base 'A'
void make_sequences(Sites &s, const SitesMapping &m, awg_arg_input &in) {
    for (size_t i = 0; i < s.positions.size(); i++) s.positions[i] = m.dst_col[i];
    s.start_coord = m.dst_start;
    s.end_coord = m.dst_end;
    const int nseqs = (int)s.names.size(), L = s.end_coord - s.start_coord;
    in.names = s.names;
    in.chrom = s.chrom;
    in.seqlen = L;
    in.start_coord = s.start_coord;
    in.seqs.assign((size_t)nseqs * L, 'A');
    const int nsites = (int)s.positions.size();
    for (int i = 0; i < nseqs; i++) {
        int col = 0;
        for (int j = 0; j < L; j++)
            if (col < nsites && s.start_coord + j == s.positions[col])
                in.seqs[(size_t)i * L + j] = s.cols[col++][i];
    }
}

// ------------------------------------------------------------------------- SMC

// find_time (local_tree.cpp:1022-1036): the closest time point, the first on ties
int find_time(double t, const std::vector<double> &times) {
    double mindiff = INFINITY;
    int mini = -1;
    for (int i = 0; i < (int)times.size(); i++) {
        const double diff = fabs(times[i] - t);
        if (diff < mindiff) {
            mindiff = diff;
            mini = i;
        }
    }
    return mini;
}

// the "age" value of an NHX comment text[0..len) ("&&NHX:key=value:..."; parse_node_age,
// local_tree.cpp:1064-1090)
bool nhx_age(const char *text, int len, double *age) {
    if (len < 6 || strncmp(text, "&&NHX:", 6) != 0) return false;
    int k = 6;
    while (k < len) {
        int ke = k;
        while (ke < len && text[ke] != '=') ke++;
        if (ke >= len) return false;
        int v = ke + 1, ve = v;
        while (ve < len && text[ve] != ':') ve++;
        if (ke - k == 3 && strncmp(text + k, "age", 3) == 0) {
            const std::string val(text + v, text + ve);
            return sscanf(val.c_str(), "%lf", age) == 1;
        }
        k = ve + 1;
    }
    return false;
}

struct PTree {
    std::vector<int> parent, age, c0, c1;
    int root = -1;
};

// parse_local_tree (local_tree.cpp:1094-1231): nodes named by integers, ages from NHX
// "age" comments snapped to the time grid; leaves without an age are at time 0
bool parse_tree(const std::string &nw, int nnodes, const std::vector<double> &times, PTree &t) {
    const int len = (int)nw.size();
    std::vector<int> ptree{-1}, ages{-1}, names{-1}, stack;
    int node = 0;
    for (int i = 0; i < len; i++) {
        const char ch = nw[i];
        if (ch == '(') {
            ptree.push_back(node); ages.push_back(-1); names.push_back(-1);
            stack.push_back(node);
            node = (int)ptree.size() - 1;
        } else if (ch == ',') {
            if (stack.empty()) return false;
            ptree.push_back(stack.back()); ages.push_back(-1); names.push_back(-1);
            node = (int)ptree.size() - 1;
        } else if (ch == ')') {
            if (stack.empty()) return false;
            node = stack.back();
            stack.pop_back();
        } else if (ch == ':' || ch == ';') {
        } else if (ch == '[') {
            int j = i + 1;
            while (j < len && nw[j] != ']') j++;
            if (j >= len) return false;
            double age;
            if (nhx_age(nw.c_str() + i + 1, j - i - 1, &age)) ages[node] = find_time(age, times);
            i = j;
        } else {
            const char last = i > 0 ? nw[i - 1] : '(';
            while (i < len && nw[i] == ' ') i++;
            int j = i;
            while (j < len && !strchr(")(,:;[", nw[j])) j++;
            if (last == ')' || last == '(' || last == ',') {
                if (sscanf(nw.c_str() + i, "%d", &names[node]) != 1) return false;
            }
            i = j - 1;
        }
    }
    if (!stack.empty()) return false;
    const int n = (int)ptree.size();
    if (n != nnodes) return false;
    t.parent.assign(n, -1); t.age.assign(n, -1); t.c0.assign(n, -1); t.c1.assign(n, -1);
    std::vector<char> seen(n, 0);
    for (int i = 0; i < n; i++) {
        const int j = names[i];
        if (j < 0 || j >= n || seen[j]) return false;
        seen[j] = 1;
    }
    for (int i = 0; i < n; i++) {
        const int j = names[i];
        t.parent[j] = ptree[i] != -1 ? names[ptree[i]] : -1;
        if (ptree[i] == -1) t.root = j;
        t.age[j] = ages[i];
    }
    for (int i = 0; i < n; i++) {  // add_child in document order
        if (ptree[i] == -1) continue;
        const int p = names[ptree[i]], c = names[i];
        if (t.c0[p] == -1) t.c0[p] = c;
        else if (t.c1[p] == -1) t.c1[p] = c;
        else return false;
    }
    for (int i = 0; i < n; i++) {
        if (t.c0[i] == -1 && t.age[i] == -1) t.age[i] = 0;
        if (t.age[i] < 0) return false;
        if ((t.c0[i] == -1) != (t.c1[i] == -1)) return false;
    }
    return true;
}

struct SmcTrees {
    std::vector<std::string> names;
    std::string chrom;
    int start_coord = 0, end_coord = 0;
    std::vector<PTree> trees;
    std::vector<int> blocklens;
    std::vector<int> spr;  // [ntrees][4]: the SPR into each tree (-1 for the first)
};

// read_local_trees (local_tree.cpp:1422-1540)
bool read_smc(FILE *f, const std::vector<double> &times, SmcTrees &s) {
    std::string line;
    int nnodes = 0, lineno = 0;
    int spr[4] = {-1, -1, -1, -1};
    while (get_line(f, line)) {
        lineno++;
        const std::string at = " (line " + std::to_string(lineno) + ")";
        if (line.compare(0, 5, "NAMES") == 0) {
            s.names = split_tabs(line.size() > 6 ? line.substr(6) : std::string());
            nnodes = 2 * (int)s.names.size() - 1;
        } else if (line.compare(0, 5, "RANGE") == 0) {
            fail("smc: deprecated RANGE line (use REGION)" + at);
            return false;
        } else if (line.compare(0, 7, "REGION\t") == 0) {
            char chrom[51];
            if (sscanf(line.c_str() + 7, "%50s\t%d\t%d", chrom, &s.start_coord, &s.end_coord) != 3) {
                fail("smc: bad REGION line" + at);
                return false;
            }
            s.chrom = chrom;
            s.start_coord--;
        } else if (line.compare(0, 4, "TREE") == 0) {
            int start, end;
            if (line.size() < 5 || sscanf(line.c_str() + 5, "%d\t%d", &start, &end) != 2) {
                fail("smc: bad TREE line" + at);
                return false;
            }
            size_t p = line.find('\t', 5);
            p = p == std::string::npos ? p : line.find('\t', p + 1);
            if (p == std::string::npos) {
                fail("smc: bad TREE line" + at);
                return false;
            }
            PTree t;
            if (!parse_tree(line.substr(p + 1), nnodes, times, t)) {
                fail("smc: bad newick tree" + at);
                return false;
            }
            s.trees.push_back(t);
            s.blocklens.push_back(end - start + 1);
            for (int k = 0; k < 4; k++) s.spr.push_back(s.trees.size() == 1 ? -1 : spr[k]);
        } else if (line.compare(0, 3, "SPR") == 0) {
            int pos;
            double rt, ct;
            if (line.size() < 4 ||
                sscanf(line.c_str() + 4, "%d\t%d\t%lf\t%d\t%lf", &pos, &spr[0], &rt, &spr[2], &ct) != 5) {
                fail("smc: bad SPR line" + at);
                return false;
            }
            spr[1] = find_time(rt, times);
            spr[3] = find_time(ct, times);
        }
    }
    if (s.trees.empty()) {
        fail("smc: no TREE lines");
        return false;
    }
    return true;
}

}  // namespace

namespace awg {

bool read_smc_arrays(const char *path, const double *times, int ntimes, SmcArrays &out,
                     std::string &err) {
    if (!path || !times || ntimes < 2) {
        err = "read_local_trees: bad arguments";
        return false;
    }
    SmcTrees s;
    {
        Stream st(path, false);
        if (!st.f) {
            err = std::string("cannot read SMC file '") + path + "'";
            return false;
        }
        if (!read_smc(st.f, std::vector<double>(times, times + ntimes), s)) {
            err = f_err;
            return false;
        }
    }
    const int n = 2 * (int)s.names.size() - 1, B = (int)s.trees.size();
    out.ntrees = B;
    out.nnodes = n;
    out.start_coord = s.start_coord;
    out.blocklens = s.blocklens;
    out.sprs = s.spr;
    for (int b = 0; b < B; b++) {
        const PTree &t = s.trees[b];
        if ((int)t.parent.size() != n) {
            err = "read_local_trees: a tree with the wrong number of nodes";
            return false;
        }
        out.ptrees.insert(out.ptrees.end(), t.parent.begin(), t.parent.end());
        out.ages.insert(out.ages.end(), t.age.begin(), t.age.end());
        out.c0.insert(out.c0.end(), t.c0.begin(), t.c0.end());
        out.c1.insert(out.c1.end(), t.c1.begin(), t.c1.end());
    }
    return true;
}

}  // namespace awg

extern "C" {

const char *awg_formats_last_error(void) { return f_err.c_str(); }

awg_arg_input *awg_read_arg_input(const char *sites_path, const char *smc_path, int compress,
                                  const double *times, int ntimes) {
    f_err.clear();
    if (!sites_path || compress < 1 || (smc_path && (!times || ntimes < 2))) {
        fail("awg_read_arg_input: bad arguments");
        return nullptr;
    }
    Sites sites;
    {
        Stream st(sites_path, false);
        if (!st.f) {
            fail(std::string("cannot read sites file '") + sites_path + "'");
            return nullptr;
        }
        if (!read_sites(st.f, sites, -1, -1)) return nullptr;
    }
    SitesMapping mp;
    if (!find_compress_cols(sites, compress, mp)) {
        fail("sites: cannot compress by that factor (too many variant sites)");
        return nullptr;
    }
    awg_arg_input *in = new awg_arg_input();
    make_sequences(sites, mp, *in);
    if (!smc_path) return in;

    SmcTrees s;
    const std::vector<double> tv(times, times + ntimes);
    {
        Stream st(smc_path, false);
        if (!st.f) {
            fail(std::string("cannot read SMC file '") + smc_path + "'");
            delete in;
            return nullptr;
        }
        if (!read_smc(st.f, tv, s)) {
            delete in;
            return nullptr;
        }
    }
    const int nleaves = (int)s.names.size(), nnodes = 2 * nleaves - 1, B = (int)s.trees.size();
    // set_seqids (local_tree.h:603-622): SMC leaf i is sequence seqids[i]
    std::vector<int> seqids(nleaves, -1);
    for (int i = 0; i < nleaves; i++) {
        for (size_t j = 0; j < in->names.size(); j++)
            if (s.names[i] == in->names[j]) {
                seqids[i] = (int)j;
                break;
            }
        if (seqids[i] < 0 || seqids[i] >= nleaves) {
            fail("SMC leaf '" + s.names[i] + "' is not among the first sequences of the sites file");
            delete in;
            return nullptr;
        }
    }
    {
        std::vector<char> used(nleaves, 0);
        for (int i = 0; i < nleaves; i++) {
            if (used[seqids[i]]) {
                fail("SMC: two leaves name the same sequence");
                delete in;
                return nullptr;
            }
            used[seqids[i]] = 1;
        }
    }
    // compress_local_trees (local_tree.cpp:818-850, fuzzy) over compress_blocks
    // (sequences.h:300-322)
    std::vector<int> bl2;
    {
        int cur = mp.dst_start;
        const int new_seqlen = mp.dst_end - mp.dst_start;
        int end = mp.src_start;
        for (int b = 0; b < B; b++) {
            end += s.blocklens[b];
            if (end < mp.src_end) {
                int cur2 = cur;
                while (cur2 < new_seqlen && mp.kept_pos[cur2] < end) cur2++;
                bl2.push_back(cur2 - cur);
                cur = cur2;
            } else {
                bl2.push_back(mp.dst_end - cur);
            }
        }
        for (int b = 0; b < B; b++)
            if (bl2[b] <= 0) {
                if (b == B - 1) {
                    fail("SMC: the last block compresses to no columns");
                    delete in;
                    return nullptr;
                }
                const int diff = 1 - bl2[b];
                bl2[b] += diff;
                bl2[b + 1] -= diff;
            }
    }
    // leaves permuted to sequence order (get_local_trees_ptrees, local_tree.cpp:1846-1890)
    std::vector<int> perm(nnodes);
    for (int i = 0; i < nnodes; i++) perm[i] = i < nleaves ? seqids[i] : i;
    in->ntrees = B;
    in->nnodes = nnodes;
    in->ptrees.assign((size_t)B * nnodes, -1);
    in->ages.assign((size_t)B * nnodes, 0);
    in->sprs.assign((size_t)B * 4, -1);
    in->blocklens = bl2;
    for (int b = 0; b < B; b++) {
        const PTree &t = s.trees[b];
        for (int j = 0; j < nnodes; j++) {
            const int p = t.parent[j];
            in->ptrees[(size_t)b * nnodes + perm[j]] = p == -1 ? -1 : perm[p];
            in->ages[(size_t)b * nnodes + perm[j]] = t.age[j];
        }
        if (b > 0) {
            const int *sp = &s.spr[(size_t)b * 4];
            if (sp[0] < 0 || sp[0] >= nnodes || sp[2] < 0 || sp[2] >= nnodes) {
                fail("SMC: an SPR names a node out of range");
                delete in;
                return nullptr;
            }
            in->sprs[(size_t)b * 4 + 0] = perm[sp[0]];
            in->sprs[(size_t)b * 4 + 1] = sp[1];
            in->sprs[(size_t)b * 4 + 2] = perm[sp[2]];
            in->sprs[(size_t)b * 4 + 3] = sp[3];
        }
    }
    return in;
}

int awg_arg_input_dims(const awg_arg_input *in, int *nseqs, int *seqlen, int *ntrees,
                       int *nnodes, int *start_coord) {
    if (!in) return -1;
    if (nseqs) *nseqs = (int)in->names.size();
    if (seqlen) *seqlen = in->seqlen;
    if (ntrees) *ntrees = in->ntrees;
    if (nnodes) *nnodes = in->nnodes;
    if (start_coord) *start_coord = in->start_coord;
    return 0;
}

const char *awg_arg_input_name(const awg_arg_input *in, int i) {
    if (!in || i < 0 || i >= (int)in->names.size()) return nullptr;
    return in->names[i].c_str();
}

int awg_arg_input_copy(const awg_arg_input *in, char *seqs, int *ptrees, int *ages, int *sprs,
                       int *blocklens) {
    if (!in) return -1;
    if (seqs) memcpy(seqs, in->seqs.data(), in->seqs.size());
    const size_t tn = (size_t)in->ntrees * in->nnodes;
    if (ptrees && tn) memcpy(ptrees, in->ptrees.data(), sizeof(int) * tn);
    if (ages && tn) memcpy(ages, in->ages.data(), sizeof(int) * tn);
    if (sprs && in->ntrees) memcpy(sprs, in->sprs.data(), sizeof(int) * 4 * in->ntrees);
    if (blocklens && in->ntrees) memcpy(blocklens, in->blocklens.data(), sizeof(int) * in->ntrees);
    return 0;
}

void awg_free_arg_input(awg_arg_input *in) { delete in; }

// write_sites (sequences.cpp:133-157): NAMES, REGION (1-based), then every column whose
// bases differ, at its 1-based position start_coord + column + 1
int awg_write_sites(const char *path, const char *const *names, int nseqs, const char *chrom,
                    int start_coord, int seqlen, const char *seqs) {
    f_err.clear();
    if (!path || !names || !chrom || !seqs || nseqs < 1 || seqlen < 0) {
        fail("awg_write_sites: bad arguments");
        return -1;
    }
    Stream st(path, true);
    if (!st.f) {
        fail(std::string("cannot write '") + path + "'");
        return -2;
    }
    fprintf(st.f, "NAMES");
    for (int i = 0; i < nseqs; i++) fprintf(st.f, "\t%s", names[i]);
    fprintf(st.f, "\nREGION\t%s\t%d\t%d\n", chrom, start_coord + 1, start_coord + seqlen);
    std::string col(nseqs, 'N');
    for (int j = 0; j < seqlen; j++) {
        bool diff = false;
        for (int i = 0; i < nseqs; i++) {
            col[i] = seqs[(size_t)i * seqlen + j];
            diff |= col[i] != col[0];
        }
        if (diff) fprintf(st.f, "%d\t%s\n", start_coord + j + 1, col.c_str());
    }
    return st.close() == 0 ? 0 : -3;
}

// write_local_trees (local_tree.cpp:1286-1362) for trees whose node numbering follows the
// default mapping (each tree's nodes keep the previous tree's numbers; the broken node is
// the recoalescence node): nodes are written by their own numbers, leaves named by
// `names`, ages as NHX comments, one SPR line between trees.
int awg_write_smc(const char *path, const char *const *names, const char *chrom,
                  int start_coord, const int *ptrees, const int *ages, const int *sprs,
                  const int *blocklens, int ntrees, int nnodes, const double *times,
                  int ntimes) {
    f_err.clear();
    if (!path || !names || !chrom || !ptrees || !ages || !blocklens || !times || ntrees < 1 ||
        nnodes < 1 || (ntrees > 1 && !sprs)) {
        fail("awg_write_smc: bad arguments");
        return -1;
    }
    const int nleaves = (nnodes + 1) / 2;
    for (size_t i = 0; i < (size_t)ntrees * nnodes; i++)
        if (ages[i] < 0 || ages[i] >= ntimes || ptrees[i] < -1 || ptrees[i] >= nnodes) {
            fail("awg_write_smc: an age or a parent out of range");
            return -1;
        }
    Stream st(path, true);
    if (!st.f) {
        fail(std::string("cannot write '") + path + "'");
        return -2;
    }
    long long total = 0;
    for (int b = 0; b < ntrees; b++) total += blocklens[b];
    fprintf(st.f, "NAMES");
    for (int i = 0; i < nleaves; i++) fprintf(st.f, "\t%s", names[i]);
    fprintf(st.f, "\nREGION\t%s\t%d\t%lld\n", chrom, start_coord + 1, start_coord + total);
    long long end = start_coord;
    std::vector<int> c0(nnodes), c1(nnodes);
    for (int b = 0; b < ntrees; b++) {
        const int *par = ptrees + (size_t)b * nnodes, *age = ages + (size_t)b * nnodes;
        const long long start = end;
        end += blocklens[b];
        std::fill(c0.begin(), c0.end(), -1);
        std::fill(c1.begin(), c1.end(), -1);
        int root = -1;
        for (int i = 0; i < nnodes; i++) {
            const int p = par[i];
            if (p == -1) root = i;
            else if (c0[p] == -1) c0[p] = i;
            else c1[p] = i;
        }
        fprintf(st.f, "TREE\t%lld\t%lld\t", start + 1, end);
        // newick with node numbers as names (the NAMES line names the leaves), children in
        // index order, as write_newick_node (local_tree.cpp:868-921) writes it
        std::function<void(int)> node = [&](int v) {
            if (c0[v] == -1) {
                fprintf(st.f, "%d", v);
            } else {
                fprintf(st.f, "(");
                node(c0[v]);
                fprintf(st.f, ",");
                node(c1[v]);
                fprintf(st.f, ")%d", v);
            }
            if (v != root) fprintf(st.f, ":%f", times[age[par[v]]] - times[age[v]]);
            fprintf(st.f, "[&&NHX:age=%f]", times[age[v]]);
        };
        node(root);
        fprintf(st.f, ";\n");
        if (b + 1 < ntrees) {
            const int *sp = sprs + (size_t)(b + 1) * 4;
            if (sp[1] < 0 || sp[1] >= ntimes || sp[3] < 0 || sp[3] >= ntimes) {
                fail("awg_write_smc: an SPR time out of range");
                return -1;
            }
            fprintf(st.f, "SPR\t%lld\t%d\t%f\t%d\t%f\n", end, sp[0], times[sp[1]], sp[2],
                    times[sp[3]]);
        }
    }
    return st.close() == 0 ? 0 : -3;
}

}  // extern "C"

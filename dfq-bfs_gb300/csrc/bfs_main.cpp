// bfs - drop-in replacement for the reference DFQ-BFS programs.
//
//   bfs <graph> [source] [options] [$]
//
// Same input, source selection, stdin prompts and per-run stdout block as
// design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu:181-317 (below "DFQ"):
//   * <graph>: the reference's .dat ("N E SOURCE", N "start length", E "dst x",
//     DFQ:187-199) or the SNAP edge list its README documents (README.md:19-32),
//     sniffed from the first byte; also the binary CSR cache (--save-bin).
//   * source: the .dat header's (DFQ:188), or 0 for SNAP.  A numeric second
//     argument overrides it (the reference ignores argv[2]; plot.py passes "8",
//     plot.py:32 - give --ref-compat to ignore it the same way).
//   * a last argument starting with '$' turns on the interactive loop: after
//     each run "Exit? [y/n]" then "Source  : " read from stdin (DFQ:202-214,302-308).
//   * stdout per run: "# Nodes : N", "# Edges : E", "Source  : S", "- Dist  = d",
//     "- Touch = p % (r / N)", "- Error = k", "- Time  = <ms>ms" (DFQ:206-208,297-300),
//     then "\033[0m" at exit (DFQ:311).  The time stays the second-to-last
//     whitespace token, which is what plot.py parses (plot.py:33).
//   * "- Error" counts vertices whose level differs from a serial CPU BFS run
//     by this program (the reference's self-check, DFQ:218-253,290-296); this
//     program also counts vertices reached on the GPU but not on the CPU.
#include "dfq.h"

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

bool is_int(const char* s) {
    if (!*s) return false;
    for (const char* p = (*s == '-' ? s + 1 : s); *p; ++p)
        if (*p < '0' || *p > '9') return false;
    return true;
}
bool is_int_prefix(const char* s) { return is_int(s) && strlen(s) < 11; }

void usage() {
    fprintf(stderr,
            "usage: bfs <graph> [source] [--ref-compat] [--symmetrize] [--parents] [--no-check]\n"
            "           [--repeat K] [--autotune] [--json] [--save-bin PATH] [--opt NAME=VALUE]...\n"
            "           [--frontier-profile [--profile-tiles A,B,C,E] [--profile-grid BLOCKS]] [$]\n"
            "  --opt sets one field of dfq_opts (include/dfq.h), e.g. --opt probe_first=0;\n"
            "  the reference's design variants are separate programs, here they are options\n"
            "  --frontier-profile prints the reference profiler's idle lanes per level and bin\n"
            "  (bfs_ftr_prof.cu; tiles default 16,128,1024,8192, grid 304 blocks of 1024)\n");
}

// dfq_opts fields settable with --opt NAME=VALUE.
struct OptField {
    const char* name;
    int32_t dfq_opts::*field;
};
const OptField kOptFields[] = {
    {"block_threads", &dfq_opts::block_threads},       {"blocks_per_sm", &dfq_opts::blocks_per_sm},
    {"medium_min_degree", &dfq_opts::medium_min_degree}, {"large_min_degree", &dfq_opts::large_min_degree},
    {"local_queue_cap", &dfq_opts::local_queue_cap},   {"local_edge_budget", &dfq_opts::local_edge_budget},
    {"piece_edges", &dfq_opts::piece_edges},           {"probe_first", &dfq_opts::probe_first},
    {"l2_persist", &dfq_opts::l2_persist},             {"use_tma", &dfq_opts::use_tma},
    {"timeout_ms", &dfq_opts::timeout_ms},             {"hot_cache", &dfq_opts::hot_cache},
    {"vertex_order", &dfq_opts::vertex_order},         {"direction", &dfq_opts::direction},
    {"cluster_blocks", &dfq_opts::cluster_blocks},
};

// Apply "NAME=VALUE" to o; false if the name or the value is not recognised.
bool set_opt(dfq_opts& o, const char* kv) {
    const char* eq = strchr(kv, '=');
    if (!eq || !is_int_prefix(eq + 1)) return false;
    for (const OptField& f : kOptFields)
        if (strlen(f.name) == (size_t)(eq - kv) && !strncmp(f.name, kv, eq - kv)) {
            o.*(f.field) = (int32_t)atoi(eq + 1);
            return true;
        }
    return false;
}


// The reference's serial CPU BFS (DFQ:218-253): frontier walked back to front.
void cpu_bfs(const dfq_csr& g, int32_t src, std::vector<int32_t>& lv) {
    lv.assign(g.n, -1);
    std::vector<int32_t> F{src}, Fn;
    lv[src] = 0;
    while (!F.empty()) {
        Fn.clear();
        for (int64_t i = (int64_t)F.size() - 1; i >= 0; --i) {
            const int32_t id = F[i];
            for (int32_t j = g.offsets[id]; j < g.offsets[id + 1]; ++j) {
                const int32_t nid = g.cols[j];
                if (lv[nid] < 0) { lv[nid] = lv[id] + 1; Fn.push_back(nid); }
            }
        }
        F.swap(Fn);
    }
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) { usage(); return 2; }
    const char* path = argv[1];
    bool ref_compat = false, symmetrize = false, want_parents = false, check = true, json = false,
         autotune = false;
    int repeat = 1;
    const char* save_bin = nullptr;
    bool frontier_profile = false;
    int32_t prof_tiles[4] = {16, 128, 1024, 8192};  // the reference profiler's TILE_SIZ_A/B/C/E
    int32_t prof_grid = 304;                          // its occupancy-sized grid on GB300 (x 1024 threads)
    long long src_arg = -1;
    const bool interactive = argv[argc - 1][0] == '$';
    dfq_opts opts;
    dfq_opts_default(&opts);
    for (int i = 2; i < argc; ++i) {
        const char* a = argv[i];
        if (interactive && i == argc - 1) continue;
        if (!strcmp(a, "--ref-compat")) ref_compat = true;
        else if (!strcmp(a, "--symmetrize")) symmetrize = true;
        else if (!strcmp(a, "--parents")) want_parents = true;
        else if (!strcmp(a, "--no-check")) check = false;
        else if (!strcmp(a, "--json")) json = true;
        else if (!strcmp(a, "--autotune")) autotune = true;
        else if (!strcmp(a, "--repeat") && i + 1 < argc) repeat = atoi(argv[++i]);
        else if (!strcmp(a, "--save-bin") && i + 1 < argc) save_bin = argv[++i];
        else if (!strcmp(a, "--frontier-profile")) frontier_profile = true;
        else if (!strcmp(a, "--profile-tiles") && i + 1 < argc) {
            int t[4];
            char tail = 0;
            bool ok = sscanf(argv[++i], "%d,%d,%d,%d%c", &t[0], &t[1], &t[2], &t[3], &tail) == 4;
            for (int k = 0; ok && k < 4; ++k)
                ok = t[k] > 0 && (t[k] & (t[k] - 1)) == 0 && (k == 0 || t[k] > t[k - 1]);
            if (!ok) {
                fprintf(stderr, "bfs: --profile-tiles '%s': need four increasing powers of two A,B,C,E\n", argv[i]);
                return 2;
            }
            for (int k = 0; k < 4; ++k) prof_tiles[k] = t[k];
        }
        else if (!strcmp(a, "--profile-grid") && i + 1 < argc) {
            prof_grid = atoi(argv[++i]);
            if (prof_grid < 1) { fprintf(stderr, "bfs: --profile-grid needs a block count >= 1\n"); return 2; }
        }
        else if (!strcmp(a, "--opt") && i + 1 < argc) {
            if (!set_opt(opts, argv[++i])) {
                fprintf(stderr, "bfs: --opt '%s': not NAME=INTEGER with a dfq_opts field name\n", argv[i]);
                return 2;
            }
        }
        else if (i == 2 && is_int(a)) src_arg = atoll(a);
        else if (!strcmp(a, "-h") || !strcmp(a, "--help")) { usage(); return 0; }
        else { fprintf(stderr, "bfs: unknown argument '%s'\n", a); usage(); return 2; }
    }
    if (repeat < 1) repeat = 1;

    // banner: the reference prints argv[1] + 15 (DFQ:183), undefined for
    // shorter paths; here shorter paths print their base name
    const size_t plen = strlen(path);
    const char* banner = plen > 15 ? path + 15 : (strrchr(path, '/') ? strrchr(path, '/') + 1 : path);
    printf("\033[0;1;33m%s\033[0;1m\n", banner);
    fflush(stdout);

    dfq_csr g;
    int rc = dfq_csr_load(path, DFQ_FMT_AUTO, symmetrize ? DFQ_CSR_SYMMETRIZE : 0, &g);
    if (rc) { fprintf(stderr, "bfs: %s\n", dfq_last_error()); printf("\033[0m"); return 1; }
    if (save_bin && dfq_csr_save(save_bin, &g, DFQ_FMT_BIN))
        fprintf(stderr, "bfs: --save-bin: %s\n", dfq_last_error());
    int32_t source = g.source;
    if (src_arg >= 0 && !ref_compat) source = (int32_t)src_arg;

    dfq_graph* dg = nullptr;
    rc = dfq_graph_create(g.offsets, g.cols, g.n, g.e, &opts, &dg);
    if (rc) { fprintf(stderr, "bfs: %s\n", dfq_last_error()); printf("\033[0m"); dfq_csr_free(&g); return 1; }

    std::vector<int32_t> levels(g.n), parents(want_parents ? g.n : 0), cpu;
    std::string is_exit;
    int status = 0;
    while (is_exit != "y") {
        do {
            if (is_exit.empty()) {
                printf("# Nodes : %d\n# Edges : %lld\nSource  : %d\n", g.n, (long long)g.e, source);
            } else {
                printf("Source  : ");
                fflush(stdout);
                long long s;
                if (scanf("%lld", &s) != 1) { is_exit = "y"; break; }
                source = (int32_t)(s < INT32_MIN ? INT32_MIN : s > INT32_MAX ? INT32_MAX : s);
            }
        } while (source >= g.n || source < 0);
        if (is_exit == "y") break;
        if (autotune) {
            dfq_opts best;
            if (dfq_autotune(dg, &source, 1, &best)) fprintf(stderr, "bfs: autotune: %s\n", dfq_last_error());
            autotune = false;
        }
        dfq_stats st;
        std::vector<float> times;
        for (int r = 0; r < repeat && rc == DFQ_OK; ++r) {
            rc = dfq_bfs(dg, source, levels.data(), want_parents ? parents.data() : nullptr, &st);
            times.push_back(st.kernel_ms);
        }
        if (rc) { fprintf(stderr, "bfs: %s\n", dfq_last_error()); status = 1; break; }
        int64_t near_nodes = 0, near_errors = 0, extra = 0;
        int32_t dist = 0;
        if (check) {
            cpu_bfs(g, source, cpu);
            for (int32_t i = 0; i < g.n; ++i) {
                if (cpu[i] >= 0) {
                    ++near_nodes;
                    if (levels[i] != cpu[i]) ++near_errors;
                    else if (levels[i] > dist) dist = levels[i];
                } else if (levels[i] != -1) {
                    ++extra;
                }
            }
        } else {
            for (int32_t i = 0; i < g.n; ++i)
                if (levels[i] >= 0) { ++near_nodes; if (levels[i] > dist) dist = levels[i]; }
        }
        int64_t tree_bad = 0;
        if (want_parents) {  // every parent edge exists and spans exactly one level
            for (int32_t v = 0; v < g.n; ++v) {
                const int32_t p = parents[v];
                if (v == source) { tree_bad += (p != v); continue; }
                if (levels[v] < 0) { tree_bad += (p != -1); continue; }
                bool okp = p >= 0 && p < g.n && levels[p] == levels[v] - 1;
                if (okp) {
                    okp = false;
                    for (int32_t j = g.offsets[p]; j < g.offsets[p + 1]; ++j)
                        if (g.cols[j] == v) { okp = true; break; }
                }
                tree_bad += !okp;
            }
        }
        const int64_t errors = near_errors + extra + tree_bad;
        if (frontier_profile) {
            // the reference profiler's block (bfs_ftr_prof.cu:110-114,206-208), before the result
            // lines so that "- Time" stays the second-to-last token
            const int64_t threads = (int64_t)prof_grid * 1024;
            const int32_t max_levels = st.depth + 1;
            std::vector<int64_t> idle((size_t)max_levels * 5), count((size_t)max_levels * 5);
            const int k = dfq_frontier_profile(&g, levels.data(), prof_tiles, threads, max_levels, idle.data(),
                                               count.data());
            if (k < 0) {
                fprintf(stderr, "bfs: frontier profile: %s\n", dfq_last_error());
                status = 1;
            } else {
                printf("Dim: %d %d\n", prof_grid, 1024);
                printf("Siz: %d %d %d %d %lld\n", prof_tiles[0], prof_tiles[1], prof_tiles[2], prof_tiles[3],
                       (long long)threads);
                printf("Rng: %d %d %d %d inf\n", prof_tiles[0], prof_tiles[1], prof_tiles[2], prof_tiles[3]);
                for (int l = 0; l < k; ++l)
                    printf("%d: %lld %lld %lld %lld %lld\n", l, (long long)idle[(size_t)l * 5],
                           (long long)idle[(size_t)l * 5 + 1], (long long)idle[(size_t)l * 5 + 2],
                           (long long)idle[(size_t)l * 5 + 3], (long long)idle[(size_t)l * 5 + 4]);
            }
        }
        printf("- Dist  = %d\n", dist);
        printf("- Touch = %g %% (%lld / %d)\n", (double)near_nodes / (double)g.n * 100, (long long)near_nodes, g.n);
        if (errors) printf("- Error = \033[31m%lld\033[0;1m\n", (long long)errors);
        else printf("- Error = 0\n");
        printf("- Time  = %gms\n", (double)times[0]);
        if (json) {
            std::vector<float> s = times;
            std::sort(s.begin(), s.end());
            const double med = s[s.size() / 2];
            printf("{\"source\": %d, \"depth\": %d, \"reached\": %lld, \"edges\": %lld, \"ms_first\": %g, "
                   "\"ms_median\": %g, \"repeat\": %d, \"gteps\": %g, \"errors\": %lld}\n",
                   source, st.depth, (long long)st.reached, (long long)st.edges, (double)times[0], med, repeat,
                   med > 0 ? (double)st.edges / (med * 1e-3) / 1e9 : 0.0, (long long)errors);
        }
        fflush(stdout);
        if (errors) status = 1;
        if (interactive) {
            printf("\033[5mExit? [y/n]\033[0;1m ");
            fflush(stdout);
            char buf[64];
            if (scanf("%63s", buf) != 1) is_exit = "y";
            else is_exit = buf;
            printf("\033[1A\033[K");
        } else {
            is_exit = "y";
        }
    }
    printf("\033[0m");
    fflush(stdout);
    dfq_graph_destroy(dg);
    dfq_csr_free(&g);
    return status;
}

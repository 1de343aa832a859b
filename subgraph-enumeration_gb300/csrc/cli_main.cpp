// graph_mining_system — drop-in for the reference's binary of the same name
// (main.cpp:12-230, utility/command.cpp:8-56).  Same flags and log keys:
//   -q query  -d data  [-r result-log]  [-i] (exploration-style)  [-u] (IEP)
//   [-t threads]  [--help|-h]
// plus additive flags: --device N, --batch LIST (one pattern path per line,
// counted in one persistent launch), --seed S, --plan FILE (run the plan the
// reference printed: its "num bags:" block or a whole log holding it, imported
// by sge_plan_from_order_text instead of planning here) and --bags (with
// --plan: materialise the decomposition's bag relations as tries and let the
// leaf read them, sge_bags_create + sge_plan_use_bags).
// Like the reference, -r redirects the text log to a file; it also writes the
// sorted instance set to <file>.matches (<file>.<i>.matches for --batch), one
// row per instance in the row format of the reference's storeMatches
// (matching/join.cpp:1703-1711: the row count, then the ids of each row
// followed by a space).  The reference itself never writes this set.
// Labeled graphs in the reference's "t / v id label degree / e u v" text
// format are recognised by their leading 't' (data and query alike): a
// labeled query on a labeled data graph is counted with labels.
// Planning runs on the host; the join runs on the GPU through libsge.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <iostream>
#include <string>
#include <vector>

#include "sge.h"

namespace {

// A file in the labeled text format starts with 't'.
bool is_labeled_file(const std::string &path) {
    std::ifstream f(path);
    char c = 0;
    return f && (f >> c) && c == 't';
}

struct Args {
    std::string q, d, r, batch, plan;
    bool iep = false, explore = false, help = false, bags = false;
    int threads = 0, device = 0;
    unsigned long long seed = 1;
};

bool parse(int argc, char **argv, Args &a) {
    for (int i = 1; i < argc; ++i) {
        std::string s = argv[i];
        auto need = [&](std::string &dst) {
            if (i + 1 >= argc) return false;
            dst = argv[++i];
            return true;
        };
        std::string v;
        if (s == "-q") { if (!need(a.q)) return false; }
        else if (s == "-d") { if (!need(a.d)) return false; }
        else if (s == "-r") { if (!need(a.r)) return false; }
        else if (s == "-i") a.explore = true;
        else if (s == "-u") a.iep = true;
        else if (s == "-t") { if (!need(v)) return false; a.threads = atoi(v.c_str()); }
        else if (s == "--device") { if (!need(v)) return false; a.device = atoi(v.c_str()); }
        else if (s == "--batch") { if (!need(a.batch)) return false; }
        else if (s == "--seed") { if (!need(v)) return false; a.seed = strtoull(v.c_str(), nullptr, 10); }
        else if (s == "--plan") { if (!need(a.plan)) return false; }
        else if (s == "--bags") a.bags = true;
        else if (s == "-h" || s == "--help") a.help = true;
        else { std::cerr << "unknown option " << s << "\n"; return false; }
    }
    return true;
}

void usage() {
    std::cout << "Usage: graph_mining_system -q QUERY -d DATA [-r RESULT] [-i] [-u] [-t THREADS]\n"
                 "       [--device N] [--batch PATTERN_LIST] [--seed S] [--plan REFERENCE_PLAN [--bags]]\n"
                 "  -q  query graph path\n  -d  data graph path (text or BINGRPH)\n"
                 "  -r  result path (log destination)\n  -i  exploration-style intersection\n"
                 "  -u  IEP counting of the last levels\n  -t  threads (accepted; the GPU uses all SMs)\n";
}

}  // namespace

int main(int argc, char **argv) {
    Args a;
    if (!parse(argc, argv, a) || a.help || (a.q.empty() && a.batch.empty()) || a.d.empty() ||
        (!a.plan.empty() && !a.batch.empty()) || (a.bags && a.plan.empty())) {
        usage();
        return a.help ? 0 : 1;
    }
    std::string plan_text;
    if (!a.plan.empty()) {
        std::ifstream pf(a.plan);
        if (!pf) { std::cout << "Can not open file " << a.plan << "!" << std::endl; return 1; }
        plan_text.assign(std::istreambuf_iterator<char>(pf), std::istreambuf_iterator<char>());
    }
    std::ofstream file;
    if (!a.r.empty()) file.open(a.r);
    std::ostream &out = a.r.empty() ? std::cout : file;
    std::vector<std::string> queries;
    if (!a.batch.empty()) {
        std::ifstream bl(a.batch);
        if (!bl) { std::cout << "Can not open file " << a.batch << "!" << std::endl; return 1; }
        std::string line;
        while (std::getline(bl, line)) if (!line.empty()) queries.push_back(line);
    } else {
        queries.push_back(a.q);
    }
    uint32_t *off = nullptr, *nb = nullptr, *glab = nullptr, n = 0;
    uint64_t nnz = 0;
    const bool data_labeled = is_labeled_file(a.d);
    if ((data_labeled ? sge_load_labeled_graph_file(a.d.c_str(), &off, &nb, &glab, &n, &nnz)
                      : sge_load_graph_file(a.d.c_str(), &off, &nb, &n, &nnz)) != SGE_OK) {
        std::cout << sge_last_error() << std::endl;
        return 1;
    }
    sge_graph *g = nullptr;
    if (sge_graph_create(off, nb, n, nnz, a.device, &g) != SGE_OK ||
        (data_labeled && sge_graph_set_labels(g, glab) != SGE_OK)) {
        std::cout << "error: " << sge_last_error() << std::endl;
        return 1;
    }
    auto t0 = std::chrono::steady_clock::now();
    std::vector<sge_plan *> plans;
    std::vector<sge_plan_blob> blobs;
    std::vector<std::vector<uint32_t>> pedges;
    std::vector<uint32_t> pk;
    std::vector<uint32_t> nbags;
    std::vector<char> qlabeled;
    sge_bags *bags = nullptr;
    sge_graph_stats gst{};
    if (!plan_text.empty() && sge_graph_stats_compute(off, nb, n, &gst) != SGE_OK) {
        std::cout << "error: " << sge_last_error() << std::endl;
        return 1;
    }
    for (auto &qp : queries) {
        uint32_t k = 0, m = 0, edges[2 * SGE_MAX_K * SGE_MAX_K];
        uint32_t qlab[SGE_MAX_K] = {};
        const bool query_labeled = is_labeled_file(qp);
        if (query_labeled) {
            // a labeled query: its CSR back to an edge list, plus its labels
            uint32_t *qo = nullptr, *qn = nullptr, *ql = nullptr, qv = 0;
            uint64_t qnnz = 0;
            if (sge_load_labeled_graph_file(qp.c_str(), &qo, &qn, &ql, &qv, &qnnz) != SGE_OK) {
                std::cout << sge_last_error() << std::endl;
                return 1;
            }
            if (qv > SGE_MAX_K || !data_labeled) {
                std::cout << "error: " << (qv > SGE_MAX_K ? "query has too many vertices" : "labeled query on an unlabeled data graph")
                          << std::endl;
                return 1;
            }
            k = qv;
            for (uint32_t u = 0; u < qv; ++u) {
                qlab[u] = ql[u];
                for (uint32_t e = qo[u]; e < qo[u + 1]; ++e)
                    if (qn[e] > u) { edges[2 * m] = u; edges[2 * m + 1] = qn[e]; ++m; }
            }
            sge_free_host(qo);
            sge_free_host(qn);
            sge_free_host(ql);
        } else if (sge_load_pattern_file(qp.c_str(), &k, &m, edges) != SGE_OK) {
            std::cout << sge_last_error() << std::endl;
            return 1;
        }
        sge_plan_opts po{};
        po.join_style = a.explore ? SGE_JOIN_EXPLORATION : SGE_JOIN_WCOJ;
        po.use_iep = a.iep ? 1u : 0u;
        po.max_tail = SGE_MAX_TAIL;
        po.seed = a.seed;
        if (query_labeled) po.vertex_labels = qlab;
        sge_plan_blob b;
        uint32_t nb_plan = 0;
        const sge_status ps = plan_text.empty()
                                  ? sge_plan_pattern(k, m, edges, g, &po, &b)
                                  : sge_plan_from_order_text(k, m, edges, plan_text.c_str(), &gst, &po, &b, &nb_plan);
        if (ps != SGE_OK) {
            std::cout << "error: " << sge_last_error() << std::endl;
            return 1;
        }
        sge_plan *p = nullptr;
        if (sge_plan_create(&b, &p) != SGE_OK || (query_labeled && sge_plan_set_labels(p, qlab) != SGE_OK)) {
            std::cout << "error: " << sge_last_error() << std::endl;
            return 1;
        }
        if (a.bags) {
            uint32_t levels = 0;
            if (sge_bags_create(g, k, m, edges, plan_text.c_str(), 0, &bags) != SGE_OK ||
                sge_plan_use_bags(p, bags, &levels) != SGE_OK) {
                std::cout << "error: " << sge_last_error() << std::endl;
                return 1;
            }
        }
        nbags.push_back(plan_text.empty() ? (b.single_bag ? 1u : 2u) : nb_plan);
        qlabeled.push_back(query_labeled ? 1 : 0);
        blobs.push_back(b);
        plans.push_back(p);
        pedges.emplace_back(edges, edges + 2 * m);
        pk.push_back(k);
    }
    double plan_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (size_t i = 0; i < blobs.size(); ++i) {
        const sge_plan_blob &b = blobs[i];
        out << "num bags: " << nbags[i] << std::endl;
        out << "matching order:";
        for (uint32_t l = 0; l < b.k; ++l) out << (l ? "," : " ") << b.order[l];
        out << std::endl;
    }
    out << "Planning time (s): " << plan_s << std::endl;
    if (bags) {
        uint32_t nrel = 0, skipped = 0;
        uint64_t rows = 0, bytes = 0;
        sge_bags_info(bags, &nrel, &rows, &bytes, nullptr, &skipped);
        out << "bag relations: " << nrel << " (" << rows << " tuples, " << bytes << " bytes on the device)" << std::endl;
    }
    out << "traverse all level: 0" << std::endl;
    out << "use iep: " << (a.iep ? 1 : 0) << std::endl;
    if (a.threads > 1) out << "Number of threads: " << a.threads << std::endl;
    bool optimized = false;
    for (auto &b : blobs) optimized |= b.tail_len > 1;
    if (a.iep && optimized) out << "optimized traversal" << std::endl;
    std::vector<uint64_t> counts(plans.size()), inst(plans.size());
    sge_stats st{};
    auto t1 = std::chrono::steady_clock::now();
    sge_status s = sge_count(g, plans.data(), (uint32_t)plans.size(), nullptr, counts.data(), inst.data(), &st);
    double exec_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
    if (s != SGE_OK) {
        std::cout << "error: " << sge_last_error() << std::endl;
        return 1;
    }
    for (size_t i = 0; i < plans.size(); ++i) {
        if (plans.size() > 1) out << "pattern: " << queries[i] << std::endl;
        out << "Number of matches: " << counts[i] << std::endl;
        out << "Number of instances: " << inst[i] << std::endl;
    }
    out << "Number of intersections: " << st.set_ops << std::endl;
    out << "Execution Time: " << exec_s << std::endl;
    out << "GPU time (ms): " << st.kernel_ms << std::endl;
    if (!a.r.empty()) {
        for (size_t i = 0; i < plans.size(); ++i) {
            if (qlabeled[i]) {  // the instance set is written for unlabeled queries only
                out << "Matches not written (labeled query)" << std::endl;
                continue;
            }
            const uint32_t k = pk[i], m = (uint32_t)(pedges[i].size() / 2);
            sge_plan_opts po{};
            po.use_iep = 0;
            po.max_tail = 1;
            sge_plan_blob eb;
            sge_plan *ep = nullptr;
            if (sge_plan_pattern(k, m, pedges[i].data(), g, &po, &eb) != SGE_OK || sge_plan_create(&eb, &ep) != SGE_OK) {
                std::cout << "error: " << sge_last_error() << std::endl;
                return 1;
            }
            std::vector<uint32_t> rows((size_t)std::max<uint64_t>(inst[i], 1) * k);
            uint64_t n = 0;
            if (sge_match_set(g, ep, k, m, pedges[i].data(), rows.data(), inst[i], &n) != SGE_OK) {
                std::cout << "error: " << sge_last_error() << std::endl;
                return 1;
            }
            sge_plan_destroy(ep);
            const std::string path = a.r + (plans.size() > 1 ? "." + std::to_string(i) : std::string()) + ".matches";
            FILE *f = fopen(path.c_str(), "w");
            if (!f) { std::cout << "Can not create file " << path << "!" << std::endl; return 1; }
            fprintf(f, "%llu\n", (unsigned long long)n);
            for (uint64_t r = 0; r < n; ++r) {
                for (uint32_t j = 0; j < k; ++j) fprintf(f, "%u ", rows[r * k + j]);
                fputc('\n', f);
            }
            fclose(f);
            out << "Matches written: " << path << std::endl;
        }
    }
    for (auto *p : plans) sge_plan_destroy(p);
    sge_bags_destroy(bags);
    sge_graph_destroy(g);
    sge_free_host(off);
    sge_free_host(nb);
    sge_free_host(glab);
    return 0;
}

// The `ktruss` command line tool: same flags, output files and verification as the reference
// executable (main.cu:13-53, config.h), running the GB300 engine through the C ABI.
//
// Exit status: 0 on success; 0 on an unknown option or enum value and after -h, as the
// reference's parseArgs does (config.h:62-63, 216-221); 1 when a step fails where the
// reference would abort on an assert (unreadable file, self loop, verify mismatch, ...).

#include <sys/time.h>

#include <cstdio>
#include <cstdlib>
#include <string_view>

#include "ktruss_gb300.h"

namespace {

struct Timer {
    bool active;
    timeval start;
};

void start(Timer* t) {
    if (t->active) gettimeofday(&t->start, nullptr);
}

void stop_print(Timer* t, const char* what) {
    if (!t->active) return;
    timeval end;
    gettimeofday(&end, nullptr);
    double ms = (end.tv_sec - t->start.tv_sec) * 1e3 + (end.tv_usec - t->start.tv_usec) / 1e3;
    printf("%s: %f ms\n", what, ms);
}

int die(int rc) {
    fflush(stdout);
    fprintf(stderr, "ktruss: %s (%s)\n", kt_last_error(), kt_status_string(rc));
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    kt_config config;
    int rc = kt_parse_args(argc, argv, &config);
    if (rc) {
        if (*kt_last_error() && std::string_view(kt_last_error()) != "help requested")
            fprintf(stderr, "%s\n", kt_last_error());
        return 0;
    }
    Timer timer{config.verbosity >= 1, {}};

    if (timer.active) printf("Setting up\n");
    start(&timer);
    kt_coo graph, truss;
    if ((rc = kt_read_tsv(config.graph_file_name, &graph))) return die(rc);
    config.num_nodes = graph.num_nodes;
    config.num_edges = graph.num_edges;
    if ((rc = kt_coo_alloc(config.num_nodes, config.num_edges, &truss))) return die(rc);
    stop_print(&timer, "    Set up time");
    if (config.verbosity >= 1) kt_print_config(&config);

    if (timer.active) printf("Computing\n");
    start(&timer);
    if ((rc = kt_ktruss(&graph, &truss, &config))) return die(rc);
    stop_print(&timer, "    Total time");

    if (config.out_file_name) {
        if (config.verbosity >= 1) printf("Writing result to file: %s\n", config.out_file_name);
        if ((rc = kt_write_tsv(&truss, config.out_file_name))) return die(rc);
    }

    if (timer.active) printf("Verifying result\n");
    start(&timer);
    if ((rc = kt_verify(&truss, &config))) return die(rc);
    stop_print(&timer, "    Verification time");

    if (timer.active) printf("Cleaning up\n");
    start(&timer);
    kt_coo_free(&graph);
    kt_coo_free(&truss);
    stop_print(&timer, "    Clean up time");
    return 0;
}

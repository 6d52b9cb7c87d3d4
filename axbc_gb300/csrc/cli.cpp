// axbc: command-line driver with the reference's option surface
// (src/axbc2d.c:2334-2422, usage 1733-1750) over the axbc_gb300 C ABI.
//
//   axbc -p 1x1 (-f FILE -n N | -S SCALE [-E EF]) [-N rounds] [-c C] [-x X]
//        [-z 0..6] [-H 0|1] [-U] [-R 0|1] [-o PREFIX] [-s SEED] [-W WIDTH]
//
// Same defaults as the reference: -N 1, -c 1 (adaptive stop on), -x 1,
// -z 0, -H 0, graphs made undirected unless -U, srand48 seed 4343543.
// New options: -s SEED (srand48 seed), -W WIDTH (pivots per round, 1..64;
// 1 reproduces the reference's round sequence).  One GPU: -p must be 1x1;
// -m (force the 2-D multi-GPU code) is accepted and ignored.
#include <getopt.h>
#include <sys/time.h>
#include <unistd.h>

#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <vector>

#include "axbc.h"

static void die(const char *fmt, const char *arg = nullptr)
{
    fprintf(stderr, fmt, arg ? arg : "");
    exit(EXIT_FAILURE);
}

static void check(int rc, const char *what)
{
    if (rc != AXBC_OK) {
        fprintf(stderr, "%s failed: %s (%s)\n", what, axbc_status_str(rc), axbc_last_error());
        exit(EXIT_FAILURE);
    }
}

static void usage(const char *p)
{
    fprintf(stderr,
            "Usage:\n"
            "\t %s -p RxC [-o outfile] [-D] [-d] [-m] [-N <# of searches>]\n"
            "\t -> to visit a graph read from file:\n"
            "\t\t -f <graph file> -n <# vertices> [-r <start vert>]\n"
            "\t -> to visit an RMAT graph:\n"
            "\t\t -S <scale> [-E <edge factor>]\n"
            "\t Where:\n"
            "\t\t -c <C>   Bader stop constant (0: fixed number of rounds), default 1\n"
            "\t\t -x <X>   number of check vertices, default 1\n"
            "\t\t -z <0-6> pivot heuristic, default 0\n"
            "\t\t -H <0|1> 1-degree reduction, default 0\n"
            "\t\t -U       DO NOT make graph Undirected\n"
            "\t\t -R <0|1> 0 fixed seed, 1 time-based seed\n"
            "\t\t -s <S>   srand48 seed (default 4343543)\n"
            "\t\t -W <W>   pivots per batch 1..32 (default 1)\n"
            "\t\t -D to ENABLE debug information\n"
            "\t\t -d to DUMP RMAT generated graph to file\n"
            "\t\t -m accepted, ignored (one GPU)\n"
            "\t\t -a perform degree analysis\n\n",
            p);
    exit(EXIT_FAILURE);
}

static double now_s()
{
    struct timeval t;
    gettimeofday(&t, nullptr);
    return t.tv_sec + t.tv_usec * 1e-6;
}

int main(int argc, char **argv)
{
    int R = 0, C = 0, scale = 21, edgef = 16, H = 0, random = 0, debug = 0, dump = 0,
        analyze = 0, width = 1;
    int gread = -1;
    uint64_t N = 0, nbfs = 1, startv = 0;
    int64_t bader = 1, nchecks = 1, z = 0;
    int64_t seed = 4343543;
    int undirected = 1;
    const char *gfile = nullptr, *ofile = nullptr;
    int c;
    if (argc == 1) usage(argv[0]);
    while ((c = getopt(argc, argv, "o:p:amhDR:dUf:n:r:S:E:N:H:c:x:z:s:W:")) != -1) {
        switch (c) {
        case 'c': bader = strtoll(optarg, nullptr, 10); break;
        case 'x': nchecks = strtoll(optarg, nullptr, 10); break;
        case 'z': z = strtoll(optarg, nullptr, 10); break;
        case 'H':
            if (sscanf(optarg, "%d", &H) != 1) die("Invalid Heuristic Option (-H): %s\n", optarg);
            if (H >= 2 || H < 0) die("H2 and H3 are not implemented in Approx BC(-H): %s\n", optarg);
            break;
        case 'o': ofile = optarg; break;
        case 'p':
            if (sscanf(optarg, "%dx%d", &R, &C) != 2) die("Invalid proc mesh field.\n");
            break;
        case 'd': dump = 1; break;
        case 'R':
            if (sscanf(optarg, "%d", &random) != 1 || random < 0 || random > 3)
                die("Invalid random option (-R): %s\n", optarg);
            break;
        case 'D': debug = 1; break;
        case 'm': break;
        case 'f':
            if (gread == 1) die("Unexpected option -f!\n");
            gread = 0;
            gfile = optarg;
            break;
        case 'n':
            if (gread == 1) die("Unexpected option -n!\n");
            gread = 0;
            if (sscanf(optarg, "%" SCNu64, &N) != 1) die("Invalid number of vertices (-n): %s\n", optarg);
            break;
        case 'r':
            if (sscanf(optarg, "%" SCNu64, &startv) != 1) die("Invalid root vertex (-r): %s\n", optarg);
            break;
        case 'S':
            if (gread == 0) die("Unexpected option -S!\n");
            gread = 1;
            if (sscanf(optarg, "%d", &scale) != 1) die("Invalid scale (-S): %s\n", optarg);
            N = 1ull << scale;
            break;
        case 'E':
            if (gread == 0) die("Unexpected option -E!\n");
            gread = 1;
            if (sscanf(optarg, "%d", &edgef) != 1) die("Invalid edge factor (-S): %s\n", optarg);
            break;
        case 'N':
            if (sscanf(optarg, "%" SCNu64, &nbfs) != 1) die("Invalid number of bfs (-N): %s\n", optarg);
            break;
        case 'U': undirected = 0; break;
        case 'a': analyze = 1; break;
        case 's': seed = strtoll(optarg, nullptr, 10); break;
        case 'W':
            width = atoi(optarg);
            if (width < 1 || width > AXBC_MAX_WIDTH) die("Invalid batch width (-W): %s\n", optarg);
            break;
        default: usage(argv[0]);
        }
    }
    if (gread == -1) {
        gread = 1;
        N = 1ull << scale;
    }
    if ((uint64_t)nchecks > N) die("Number of vertices required is lager than N\n");
    if (z < 0 || z > 6) die("Select a strategy between 0 and 6\n");
    if (gread == 0 && (!gfile || !N))
        die("Graph file (-f) and number of vertices (-n) must be specified for file based bfs.\n");
    if (R != 1 || C != 1) die("This build runs on one GPU: the processor mesh (-p) must be 1x1.\n");
    if (startv >= N) die("Invalid start vertex.\n");
    if (random == 1) {
        struct timeval t;
        gettimeofday(&t, nullptr);
        seed = getpid() + t.tv_sec + t.tv_usec;
    }

    printf("Total number of vertices (N): %" PRIu64 "\n", N);
    if (gread == 0) printf("Reading graph from file: %s\n", gfile);
    else printf("RMAT graph scale: %d\nRMAT graph edge factor: %d\n", scale, edgef);
    printf("Number of bc rounds: %" PRIu64 "\nHEURISTICs: %s\nbatch width: %d\n", nbfs,
           H ? "1-degree reduction ON" : "OFF", width);

    double t0 = now_s();
    axbc_graph *g = nullptr;
    if (gread == 0) {
        uint64_t *ed = nullptr, ned = 0;
        check(axbc_read_edge_file(gfile, N, &ed, &ned), "read graph");
        uint32_t *col, *row, *reach;
        uint64_t m, removed;
        check(axbc_edges_to_csc(ed, ned, N, undirected, H, &col, &row, &m, &reach, &removed),
              "graph pre-processing");
        axbc_host_free(ed);
        check(axbc_graph_create(col, row, N, m, reach, &g), "graph upload");
        printf("Edges read: %" PRIu64 "  adjacency entries: %" PRIu64 "  removed leaves: %" PRIu64 "\n",
               ned, m, removed);
        axbc_host_free(col);
        axbc_host_free(row);
        axbc_host_free(reach);
    } else if (undirected) {
        // gen_graph (src/axbc2d.c:518-527): the Graph500 generator, seeds 23 and 24
        check(axbc_graph_generate_kronecker(scale, edgef, 23, 24, nullptr, H, &g), "graph generation");
    } else {
        // -U: the generator's pairs as directed edges, through the host pipeline
        const uint64_t ne = ((uint64_t)1 << scale) * (uint64_t)edgef;
        std::vector<int64_t> ed(2 * ne);
        check(axbc_kron_edges(scale, edgef, 23, 24, nullptr, 2, ed.data()), "graph generation");
        uint32_t *col, *row, *reach;
        uint64_t m, removed;
        check(axbc_edges_to_csc((const uint64_t *)ed.data(), ne, N, 0, H, &col, &row, &m, &reach, &removed),
              "graph pre-processing");
        check(axbc_graph_create(col, row, N, m, reach, &g), "graph upload");
        axbc_host_free(col);
        axbc_host_free(row);
        axbc_host_free(reach);
    }
    uint64_t n = 0, m = 0, bytes = 0;
    int sym = 0;
    check(axbc_graph_info(g, &n, &m, &bytes, &sym), "graph info");
    printf("Graph ready in %f secs: %" PRIu64 " vertices, %" PRIu64
           " adjacency entries, %" PRIu64 " MB on the device\n",
           now_s() - t0, n, m, bytes >> 20);
    if (dump && gread == 1) {
        char fname[256];
        snprintf(fname, sizeof fname, "rmat_S%d_EF%d.txt", scale, edgef);
        std::vector<uint32_t> col(n + 1), row(m);
        check(axbc_graph_get_csc(g, col.data(), row.data(), nullptr), "dump");
        FILE *f = fopen(fname, "w");
        if (!f) die("cannot open %s\n", fname);
        for (uint64_t v = 0; v < n; v++)
            for (uint32_t e = col[v]; e < col[v + 1]; e++) fprintf(f, "%u\t%" PRIu64 "\n", row[e], v);
        fclose(f);
        printf("DUMP THE GENERATED RMAT FILE IN %s\n", fname);
    }
    if (analyze) {
        std::vector<uint32_t> deg(n);
        check(axbc_graph_get_deg(g, deg.data()), "degrees");
        uint64_t bins[33] = {0};
        for (uint32_t d : deg) {
            int b = 0;
            while (b < 32 && (1u << b) <= d) b++;
            bins[b]++;
        }
        printf("degree histogram (bin b: 2^(b-1) <= degree < 2^b)\n");
        for (int b = 0; b <= 32; b++)
            if (bins[b]) printf("  %2d: %" PRIu64 "\n", b, bins[b]);
    }

    axbc_ctx *ctx = nullptr;
    check(axbc_ctx_create(g, nullptr, &ctx), "context");
    axbc_run_params prm;
    memset(&prm, 0, sizeof prm);
    prm.z = (int32_t)z;
    prm.bader_c = (int32_t)bader;
    prm.nbfs = nbfs;
    prm.nchecks = (uint32_t)nchecks;
    prm.H = H;
    prm.seed = seed;
    prm.batch_width = width;
    printf("task 0: BC computation is running...\ntask 0: c(bader_criterion): %" PRId64
           "\nPivot Selection Strategy: %" PRId64 "\n",
           bader, z);
    axbc_run_result res;
    double t1 = now_s();
    check(axbc_run_sampled(ctx, &prm, &res), "BC run");
    double t2 = now_s();
    if (res.stopped) printf("exit bader criterion\n");
    if (debug) {
        std::vector<uint32_t> piv(res.nrounds);
        std::vector<double> p(res.nrounds);
        uint64_t k = 0;
        check(axbc_get_pivots(ctx, piv.data(), p.data(), res.nrounds, &k), "pivots");
        for (uint64_t i = 0; i < res.nrounds; i++)
            printf("Perform %" PRIu64 "/%" PRIu64 " BC from %u (p =%lf)\n", i + 1, nbfs, piv[i], p[i]);
    }
    std::vector<float> bc(n);
    check(axbc_get_bc(ctx, bc.data()), "get_bc");
    if (ofile) {
        char fname[1024];
        snprintf(fname, sizeof fname, "%s_%dX%d_%d.log", ofile, R, C, 0);
        FILE *f = fopen(fname, "w");
        if (!f) die("cannot open %s\n", fname);
        // bc/2/nrounds, "%d\t%.2f\n" (src/axbc2d.c:3170-3176)
        for (uint64_t k = 0; k < n; k++) fprintf(f, "%d\t%.2f\n", (int)k, bc[k] / 2.0 / res.nrounds);
        fclose(f);
        printf("Result written to file: %s\n", fname);
    }
    const double secs = t2 - t1;
    printf("\n------------- RESULTS ---------------\n");
    printf("ClusterId\tSkip\tRounds\tExecTime\tRoundsTime\tMean\tTE/s\n");
    printf("%d\t%" PRIu64 "\t%" PRIu64 "\t%lf\t%lf\t%lf\t%.4g\n", 0, res.skipped, res.nrounds, secs,
           secs, res.nrounds ? secs / res.nrounds : 0.0, secs > 0 ? res.te / secs : 0.0);
    printf("task 0 BC skipped: %" PRIu64 " \ntask 0 BC rounds: %" PRIu64 "  \n", res.skipped,
           res.nrounds);
    printf("task 0 traversed edges: %" PRIu64 " in %d batches (dropped rounds %" PRIu64 ")\n",
           res.te, res.batches, res.dropped);
    axbc_ctx_destroy(ctx);
    axbc_graph_destroy(g);
    return 0;
}

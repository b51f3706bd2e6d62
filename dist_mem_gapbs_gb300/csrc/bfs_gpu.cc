// bfs_gpu — command-line drop-in for the reference's BFS binary.
//
// Same flags as CLApp (src/command_line.h:28-139, identical in gapbs-verify):
//   -f <file> -g <scale> -u <scale> -k <degree> -s -h   (CLBase, "f:g:hk:su:")
//   -a -n <trials> -r <node> -v                          (CLApp, "an:r:v")
// with the same defaults (-k 16, -n 16, random sources) and the same stdout
// lines (PrintTime / PrintStep formats of gapbs-verify/util.h; --dmm-format
// adds the "PE: 0 | " prefix of src/util.h:28-59).  Under -v each trial's
// parents are appended to bfs_output.txt in the reference's format
// (src/bfs.cc:213-235), so the reference's BFS-V checker reads it unchanged.
//
// Extra long options, which no short flag collides with:
//   --alpha <a> --beta <b>   direction-switch parameters (default 15 / 18)
//   --output <path>          file for -v (default bfs_output.txt)
//   --dmm-format             prefix every line with "PE: 0 | "
//   --sg-out <path>          write the built graph as a .sg serialized graph
//   --stepped                drive each search step by step from the host
//                            (CUDA events around every step kernel) instead of
//                            one CUDA graph launch per search

#include <getopt.h>

#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbbfs.h"

namespace {

bool g_dmm = false;

const char* prefix() { return g_dmm ? "PE: 0 | " : ""; }

void PrintLabel(const std::string& label, const std::string& val) {
  printf("%s%-21s%7s\n", prefix(), (label + ":").c_str(), val.c_str());
}
void PrintTime(const std::string& s, double seconds) {
  printf("%s%-21s%3.5lf\n", prefix(), (s + ":").c_str(), seconds);
}
void PrintStep(const std::string& s, int64_t count) {
  printf("%s%-14s%14" PRId64 "\n", prefix(), (s + ":").c_str(), count);
}
void PrintStep(const std::string& s, double seconds, int64_t count = -1) {
  if (count != -1)
    printf("%s%5s%11" PRId64 "  %10.5lf\n", prefix(), s.c_str(), count, seconds);
  else
    printf("%s%5s%23.5lf\n", prefix(), s.c_str(), seconds);
}

struct Options {
  std::string filename;
  int scale = -1;
  int degree = 16;
  bool symmetrize = false;
  bool uniform = false;
  bool analysis = false;
  int trials = 16;
  int64_t start_vertex = -1;
  bool verify = false;
  int alpha = 15, beta = 18;
  std::string output = "bfs_output.txt";
  std::string sg_out;
  bool stepped = false;
};

void Usage(const char* name) {
  auto line = [](char opt, const char* arg, const char* text, const char* def) {
    char a[32] = "", d[32] = "";
    if (arg[0]) snprintf(a, sizeof a, "<%s>", arg);
    if (def[0]) snprintf(d, sizeof d, "[%s]", def);
    printf(" -%c %-9s: %-54s%10s\n", opt, a, text, d);
  };
  printf("%s\n", name);
  line('h', "", "print this help message", "");
  line('f', "file", "load graph from file", "");
  line('s', "", "symmetrize input edge list", "false");
  line('g', "scale", "generate 2^scale kronecker graph", "");
  line('u', "scale", "generate 2^scale uniform-random graph", "");
  line('k', "degree", "average degree for synthetic graph", "16");
  line('a', "", "output analysis of last run", "false");
  line('n', "n", "perform n trials", "16");
  line('r', "node", "start from node r", "rand");
  line('v', "", "verify the output of each run", "false");
  printf("    --alpha <a> --beta <b> --output <path> --dmm-format --sg-out <path> --stepped\n");
  exit(0);
}

bool ParseArgs(int argc, char** argv, Options* o) {
  static const struct option longs[] = {
      {"alpha", required_argument, nullptr, 1000},
      {"beta", required_argument, nullptr, 1001},
      {"output", required_argument, nullptr, 1002},
      {"dmm-format", no_argument, nullptr, 1003},
      {"sg-out", required_argument, nullptr, 1004},
      {"stepped", no_argument, nullptr, 1005},
      {nullptr, 0, nullptr, 0}};
  int c;
  while ((c = getopt_long(argc, argv, "f:g:hk:su:an:r:v", longs, nullptr)) != -1) {
    switch (c) {
      case 'f': o->filename = optarg; break;
      case 'g': o->scale = atoi(optarg); break;
      case 'h': Usage("breadth-first search"); break;
      case 'k': o->degree = atoi(optarg); break;
      case 's': o->symmetrize = true; break;
      case 'u': o->uniform = true; o->scale = atoi(optarg); break;
      case 'a': o->analysis = true; break;
      case 'n': o->trials = atoi(optarg); break;
      case 'r': o->start_vertex = atol(optarg); break;
      case 'v': o->verify = true; break;
      case 1000: o->alpha = atoi(optarg); break;
      case 1001: o->beta = atoi(optarg); break;
      case 1002: o->output = optarg; break;
      case 1003: g_dmm = true; break;
      case 1004: o->sg_out = optarg; break;
      case 1005: o->stepped = true; break;
      default: return false;
    }
  }
  if (o->filename.empty() && o->scale == -1) {
    printf("No graph input specified. (Use -h for help)\n");
    return false;
  }
  if (o->scale != -1) o->symmetrize = true;  // src/command_line.h:77-78
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  Options o;
  if (!ParseArgs(argc, argv, &o)) return -1;

  int64_t *off = nullptr, n = 0, m = 0;
  int32_t* nbr = nullptr;
  gbbfs_graph* g = nullptr;
  int rc;
  if (o.scale != -1) {
    // Generated graphs: the edge list from the host generator, the CSR built
    // in HBM; the host keeps the offsets (and the neighbours for --sg-out).
    int32_t* el = nullptr;
    int64_t edges = 0;
    rc = gbbfs_generate_edges(o.scale, o.degree, o.uniform ? 1 : 0, &el, &edges);
    if (rc == GBBFS_OK) rc = gbbfs_graph_create_from_edges(el, edges, -1, &g);
    gbbfs_free_host(el);
    if (rc == GBBFS_OK) rc = gbbfs_graph_info(g, &n, &m, nullptr);
    if (rc == GBBFS_OK) {
      off = static_cast<int64_t*>(malloc(sizeof(int64_t) * (n + 1)));
      if (!o.sg_out.empty()) nbr = static_cast<int32_t*>(malloc(sizeof(int32_t) * (m + 1)));
      rc = !off || (!o.sg_out.empty() && !nbr) ? GBBFS_ERR_NOMEM
                                               : gbbfs_graph_csr(g, off, nbr);
    }
  } else {
    rc = gbbfs_read_graph(o.filename.c_str(), o.symmetrize ? 1 : 0, &off, &nbr, &n, &m);
  }
  if (rc != GBBFS_OK) {
    fprintf(stderr, "graph construction failed: %s (%s)\n", gbbfs_strerror(rc),
            gbbfs_last_error());
    return 1;
  }
  if (!o.sg_out.empty()) {
    rc = gbbfs_write_sg(o.sg_out.c_str(), off, nbr, n, m);
    if (rc != GBBFS_OK) {
      fprintf(stderr, "writing %s failed: %s\n", o.sg_out.c_str(), gbbfs_strerror(rc));
      return 1;
    }
  }
  // CSRGraph::PrintStats (src/graph.h:416-423)
  const int64_t undirected = m / 2;
  printf("%sGraph has %" PRId64 " nodes and %" PRId64 " undirected edges for degree: %" PRId64
         "\n",
         prefix(), n, undirected, undirected / n);

  if (!g) rc = gbbfs_graph_create(off, nbr, n, m, &g);
  if (rc != GBBFS_OK) {
    fprintf(stderr, "gbbfs_graph_create: %s (%s)\n", gbbfs_strerror(rc), gbbfs_last_error());
    return 1;
  }
  std::vector<int32_t> sources(o.trials > 0 ? o.trials : 1);
  rc = gbbfs_pick_sources(off, n, o.start_vertex, o.trials, sources.data());
  if (rc != GBBFS_OK) {
    fprintf(stderr, "source picking failed: %s\n", gbbfs_strerror(rc));
    return 1;
  }
  std::vector<int32_t> parent(n);
  std::vector<gbbfs_step> steps(4096);
  double total = 0, inv_teps = 0;
  int counted = 0;
  for (int t = 0; t < o.trials; t++) {
    gbbfs_stats st;
    memset(&st, 0, sizeof st);
    st.steps = steps.data();
    st.max_steps = (int32_t)steps.size();
    st.stepped = o.stepped ? 1 : 0;
    const int32_t src = sources[t];
    rc = gbbfs_bfs(g, src, o.alpha, o.beta, parent.data(), nullptr, &st);
    if (rc != GBBFS_OK) {
      fprintf(stderr, "gbbfs_bfs: %s (%s)\n", gbbfs_strerror(rc), gbbfs_last_error());
      return 1;
    }
    // DOBFS trace (gapbs-verify/bfs.cc:124-165)
    PrintStep("Source", (int64_t)src);
    PrintStep("i", st.init_seconds);
    for (int i = 0; i < st.num_steps && i < st.max_steps; i++) {
      const gbbfs_step& s = steps[i];
      switch (s.kind) {
        case GBBFS_STEP_TD: PrintStep("td", s.seconds, s.count); break;
        case GBBFS_STEP_E: PrintStep("e", s.seconds); break;
        case GBBFS_STEP_BU: PrintStep("bu", s.seconds, s.count); break;
        case GBBFS_STEP_C: PrintStep("c", s.seconds); break;
      }
    }
    const double secs = st.device_ms * 1e-3;
    PrintTime("Trial Time", secs);
    total += secs;
    // TEPS = (sum of degrees over reached vertices) / 2 / t
    int64_t degsum = 0;
    for (int64_t v = 0; v < n; v++)
      if (parent[v] >= 0) degsum += off[v + 1] - off[v];
    if (secs > 0 && degsum > 0) {
      inv_teps += secs / (degsum / 2.0);
      counted++;
    }
    if (o.analysis && t == o.trials - 1) {
      // PrintBFSStats (gapbs-verify/bfs.cc:176-187)
      int64_t tree = 0, edges = 0;
      for (int64_t v = 0; v < n; v++)
        if (parent[v] >= 0) {
          tree++;
          edges += off[v + 1] - off[v];
        }
      printf("%sBFS Tree has %" PRId64 " nodes and %" PRId64 " edges\n", prefix(), tree, edges);
    }
    if (o.verify) {
      rc = gbbfs_append_bfs_output(o.output.c_str(), parent.data(), n);
      if (rc != GBBFS_OK) {
        fprintf(stderr, "writing %s failed\n", o.output.c_str());
        return 1;
      }
    }
  }
  PrintTime("Average Time", o.trials > 0 ? total / o.trials : 0.0);
  if (counted) printf("%s%-21s%3.5lf\n", prefix(), "GTEPS (hmean):", counted / inv_teps * 1e-9);
  gbbfs_graph_destroy(g);
  gbbfs_free_host(off);
  gbbfs_free_host(nbr);
  return 0;
}

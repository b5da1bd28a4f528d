// Test program for the header-only C++ functions (include/mvkit_gb300_mv.hpp),
// written as a caller of the reference's mv::FindNccModel would write it.
//
//   mv_cpp_probe <template.raw> <tw> <th> <levels> <angle_start> <angle_extent>
//                <image.raw|-> <w> <h> <min_score> <num_matches>
// Prints the model's parameters, the exception of a search with MinScore 1.5,
// then "match row column angle score" per match of the search (an empty image
// object for "-").
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "mvkit_gb300_mv.hpp"

static std::vector<unsigned char> read_raw(const char* path) {
  std::ifstream f(path, std::ios::binary);
  return std::vector<unsigned char>(std::istreambuf_iterator<char>(f), {});
}

int main(int argc, char** argv) {
  if (argc < 12) {
    std::fprintf(stderr, "usage: see the file header\n");
    return 2;
  }
  try {
    const std::vector<unsigned char> tpl = read_raw(argv[1]);
    const mv::MvObject t = mv::GenImage1("byte", std::atoll(argv[2]), std::atoll(argv[3]), tpl.data());
    mv::MvTuple model, levels, start, extent, step, metric;
    mv::CreateNccModel(t, std::int64_t(std::atoll(argv[4])), std::atof(argv[5]), std::atof(argv[6]), "auto",
                       "use_polarity", &model);
    mv::GetNccModelParams(model, &levels, &start, &extent, &step, &metric);
    std::printf("params %lld %.17g %.17g %.17g %s\n", (long long)levels.I(), start.D(), extent.D(), step.D(),
                metric.S().c_str());
    std::vector<unsigned char> px;
    mv::MvObject image;
    if (std::string(argv[7]) != "-") {
      px = read_raw(argv[7]);
      image = mv::GenImage1("byte", std::atoll(argv[8]), std::atoll(argv[9]), px.data());
    }
    mv::MvTuple row, col, angle, score;
    try {
      mv::FindNccModel(image, model, std::atof(argv[5]), std::atof(argv[6]), 1.5, std::int64_t(1), 0.5, "true",
                       std::int64_t(0), &row, &col, &angle, &score);
      std::printf("no exception\n");
    } catch (const mv::MvException& e) {
      std::printf("exception %d %s\n", e.Status(), e.what());
    }
    mv::FindNccModel(image, model, std::atof(argv[5]), std::atof(argv[6]), std::atof(argv[10]),
                     std::int64_t(std::atoll(argv[11])), 0.5, "true", std::int64_t(0), &row, &col, &angle, &score);
    for (std::size_t i = 0; i < row.Length(); ++i)
      std::printf("match %.17g %.17g %.17g %.17g\n", row.D(i), col.D(i), angle.D(i), score.D(i));
    std::printf("count %zu\n", row.Length());
  } catch (const mv::MvException& e) {
    std::printf("failed %d %s\n", e.Status(), e.what());
    return 1;
  }
  return 0;
}

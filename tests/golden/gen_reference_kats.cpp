// Regenerates the inputs and known answers of MPPI-Generic's kernel tests whose inputs come from
// std::default_random_engine(7) (libstdc++), writing raw little-endian arrays that make_golden.py packs into npz:
//   normexp_kernel_tests.cu:45-60    baseline over 4196 costs ~ N(100, 2)          (fresh engine)
//   normexp_kernel_tests.cu:62-79    normaliser over 1024 costs, std::accumulate in double
//   normexp_kernel_tests.cu:126-150  expf(-0.3 (c - min)) over 555 costs
//   weightedreduction_kernel_tests.cu:135-172  exp costs expf(-N(5, 1.2)) with w[0] = 0, controls N(5, 1.2),
//                                     K = 1024, T = 100, C = 4, normaliser = std::accumulate in double
// The known weighted mean is written in double: sum_k (w_k / normaliser) u_k.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <numeric>
#include <random>
#include <string>
#include <vector>

template <class T>
static void dump(const std::string& dir, const char* name, const std::vector<T>& v)
{
  FILE* f = fopen((dir + "/" + name).c_str(), "wb");
  fwrite(v.data(), sizeof(T), v.size(), f);
  fclose(f);
}

int main(int argc, char** argv)
{
  const std::string dir = argc > 1 ? argv[1] : ".";
  {
    std::default_random_engine g(7.0);
    std::normal_distribution<float> d(100.0, 2.0);
    std::vector<float> c(4196);
    for (auto& x : c) x = d(g);
    dump(dir, "baseline_costs.f32", c);
    dump(dir, "baseline_known.f32", std::vector<float>{ *std::min_element(c.begin(), c.end()) });
  }
  {
    std::default_random_engine g(7.0);
    std::normal_distribution<float> d(100.0, 2.0);
    std::vector<float> c(1024);
    for (auto& x : c) x = d(g);
    dump(dir, "normalizer_costs.f32", c);
    dump(dir, "normalizer_known.f32", std::vector<float>{ (float)std::accumulate(c.begin(), c.end(), 0.0) });
  }
  {
    std::default_random_engine g(7.0);
    std::normal_distribution<float> d(100.0, 2.0);
    std::vector<float> c(555), w(555);
    for (auto& x : c) x = d(g);
    const float gamma = 0.3f;
    const float b = *std::min_element(c.begin(), c.end());
    for (int i = 0; i < 555; ++i) w[i] = expf(-gamma * (c[i] - b));
    dump(dir, "expnorm_costs.f32", c);
    dump(dir, "expnorm_known.f32", w);
  }
  {
    std::default_random_engine g(7.0);
    std::normal_distribution<float> d(5.0, 1.2);
    const int K = 1024, C = 4, T = 100;
    std::vector<float> w(K), u((size_t)C * K * T);
    for (auto& x : w) x = expf(-1 * d(g));
    w[0] = 0;
    for (auto& x : u) x = d(g);
    const float norm = (float)std::accumulate(w.begin(), w.end(), 0.0);
    std::vector<double> mean((size_t)T * C, 0.0);
    for (int k = 0; k < K; ++k)
      for (int j = 0; j < T * C; ++j) mean[j] += (double)(w[k] / norm) * (double)u[(size_t)k * T * C + j];
    dump(dir, "wr_weights.f32", w);
    dump(dir, "wr_controls.f32", u);
    dump(dir, "wr_normalizer.f32", std::vector<float>{ norm });
    dump(dir, "wr_known.f64", mean);
  }
  return 0;
}

#include "chemps2/Batch.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <exception>
#include <numeric>
#include <stdexcept>
#include <thread>

#include <cuda_runtime.h>

#include "chemps2/DMRG.h"
#include "runtime.hpp"
#include "tasks.hpp"

namespace CheMPS2 {

namespace {

// Work estimate used to start the largest problems first: sites times the largest
// bond dimension squared (the D^3 matvec cost over L sites, with D capped by the FCI
// dimension only through the scheme).
double work_estimate(const Problem* p, const ConvergenceScheme* s) {
  int dmax = 1;
  for (int i = 0; i < s->get_number(); i++) dmax = std::max(dmax, s->get_D(i));
  return static_cast<double>(p->gL()) * dmax * dmax * dmax;
}

}  // namespace

std::vector<BatchResult> SolveBatch(const std::vector<Problem*>& problems,
                                    const std::vector<ConvergenceScheme*>& schemes,
                                    const std::vector<unsigned>& seeds, int workers) {
  const size_t n = problems.size();
  if (schemes.size() != n || seeds.size() != n)
    throw std::invalid_argument("SolveBatch: problems, schemes and seeds differ in length");
  for (size_t i = 0; i < n; i++)
    if (!problems[i] || !schemes[i]) throw std::invalid_argument("SolveBatch: null problem or scheme");
  for (size_t i = 0; i < n; i++)
    for (size_t j = 0; j < i; j++)
      if (problems[i] == problems[j]) throw std::invalid_argument("SolveBatch: a Problem appears twice");

  std::vector<BatchResult> out(n);
  if (n == 0) return out;
  std::vector<size_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  workers = std::max(1, std::min<int>(workers, static_cast<int>(n)));
  if (workers > 1)
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
      return work_estimate(problems[a], schemes[a]) > work_estimate(problems[b], schemes[b]);
    });

  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) device = 0;
  std::atomic<size_t> next{0};

  auto solve_one = [&](size_t i) {
    BatchResult& r = out[i];
    const auto t0 = std::chrono::steady_clock::now();
    try {
      DMRGOptions opt;
      opt.private_seed = true;
      opt.seed = seeds[i];
      DMRG d(problems[i], schemes[i], opt);
      r.energy = d.Solve();
      r.stats = d.stats();
      r.n_matvec = r.stats.n_matvec;
      r.matvec_seconds = r.stats.t_matvec;
    } catch (const c2g::CudaError& e) {
      r.status = (e.code == cudaErrorNoDevice || e.code == cudaErrorInsufficientDriver) ? 3 : 2;
      r.error = e.what();
    } catch (const std::invalid_argument& e) {
      r.status = 1;
      r.error = e.what();
    } catch (const std::out_of_range& e) {
      r.status = 1;
      r.error = e.what();
    } catch (const std::runtime_error& e) {
      r.error = e.what();
      r.status = (r.error.find("no CUDA device") != std::string::npos) ? 3 : 4;
    } catch (const std::exception& e) {
      r.status = 4;
      r.error = e.what();
    } catch (...) {
      r.status = 4;
      r.error = "unknown error";
    }
    r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  };

  // Each worker's compilations use an equal share of the host cores among the workers
  // still solving: when the queue runs dry and workers leave, the last (largest-first
  // order: longest) problems get more compile threads.
  auto worker = [&] {
    cudaSetDevice(device);
    if (workers > 1) c2g::share_compile_threads(true);
    for (;;) {
      const size_t k = next.fetch_add(1);
      if (k >= n) break;
      solve_one(order[k]);
    }
    c2g::share_compile_threads(false);
  };

  if (workers == 1) {
    worker();
    return out;
  }
  std::vector<std::thread> pool;
  pool.reserve(workers);
  for (int w = 0; w < workers; w++) pool.emplace_back(worker);
  for (auto& t : pool) t.join();
  return out;
}

}  // namespace CheMPS2

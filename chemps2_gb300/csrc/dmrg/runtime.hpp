// Device runtime of one DMRG object: its CUDA stream, the slot table that turns task
// references into device pointers, uploaded task programs and their scratch buffers.
//
// A task Program (host/tasks.hpp) is uploaded once into one device allocation (groups,
// terms, tile list of every stage, batch table) and can then be run any number of times
// with different X / Y vectors, e.g. once per Davidson matvec. The combination stage
// (blocks that only depend on operators) runs when the program is prepared.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../device/kernels.cuh"
#include "../host/tasks.hpp"

namespace c2g {

struct CudaError : std::runtime_error {
  cudaError_t code;
  CudaError(cudaError_t c, const std::string& what) : std::runtime_error(what), code(c) {}
};

void cuda_check(cudaError_t e, const char* expr, const char* file, int line);
#define C2G_CUDA(x) ::c2g::cuda_check((x), #x, __FILE__, __LINE__)

class Runtime;

struct DevStage {
  const Group* groups = nullptr;
  const Term* terms = nullptr;
  const TileDesc* tiles = nullptr;        // item-parallel variant
  const TileDesc* tiles_large = nullptr;  // cooperative variant
  const WarpTile* tiles_warp = nullptr;   // team variant, ordered by row class
  int ngroups = 0, nterms = 0, ntiles = 0, ntiles_large = 0, ntiles_warp = 0;
  int nwarp[kWarpRowClasses] = {};        // team-variant tiles per row class
  // two-pass path of large groups: pass-1 jobs and tiles, pass-2 groups, items and tiles
  const InterJob* jobs = nullptr;
  const GemmTile* jtiles = nullptr;
  const SumGroup* sgroups = nullptr;
  const SumItem* sitems = nullptr;
  const GemmTile* stiles = nullptr;
  const int32_t* jsmall = nullptr;  // pass-1 jobs run one per warp
  int njtiles = 0, nstiles = 0, njsmall = 0;
  // The large groups in chunks of whole groups, each run as pass 1 then pass 2, so that
  // the intermediates of one chunk at a time share the intermediate buffer: ranges of
  // jtiles, jsmall and stiles.
  struct PassChunk {
    int jtile0, njtiles, small0, nsmall, stile0, nstiles;
  };
  std::vector<PassChunk> chunks;
  int64_t flops = 0, items = 0;
  std::string name;
};

struct DevProgram {
  Runtime* rt = nullptr;
  std::vector<DevStage> stages;
  const BatchEntry* entries = nullptr;
  int first_repeat = 0;
  int64_t combo_size = 0;
  int64_t flops_once = 0, flops_repeat = 0;
  int64_t nterms = 0, nentries = 0, bytes = 0;
  void* blob = nullptr;
  double* combo = nullptr;
  float* combo32 = nullptr;     // FP32 copy of the combined blocks for FP32 runs
  // sizes of the transient buffers the stages need (the runtime's shared buffers hold
  // them at run time): partial sums of split team-variant tiles and their arrival
  // counters, intermediates of the two-pass path, its split partial tiles and counters
  int64_t part_size = 0, counter_count = 0;
  int64_t inter_size = 0, gemm_part_size = 0, gemm_counter_count = 0;
  bool prepared = false;
  bool combo32_ready = false;
  DevProgram() = default;
  DevProgram(const DevProgram&) = delete;
  DevProgram& operator=(const DevProgram&) = delete;
  ~DevProgram();
};

class Runtime {
 public:
  // device < 0: the calling thread's current device (cudaGetDevice).
  explicit Runtime(int L, int device = -1);
  ~Runtime();
  Runtime(const Runtime&) = delete;
  Runtime& operator=(const Runtime&) = delete;

  cudaStream_t stream() const { return stream_; }
  // A second stream for work that overlaps the main one (created on first use), and a
  // fork / join of it with the main stream.
  cudaStream_t aux_stream();
  void fork_aux();  // aux waits for everything issued on the main stream so far
  void join_aux();  // the main stream waits for everything issued on aux so far
  // ordering with a stream of the caller: the main stream waits for what is issued on
  // `other` so far / `other` waits for what is issued on the main stream so far
  void wait_for(cudaStream_t other);
  void signal_to(cudaStream_t other);
  int L() const { return L_; }
  // the CUDA device this runtime's stream and memory belong to
  int device() const { return device_; }

  // Device memory, stream ordered on this runtime's stream.
  double* alloc(int64_t n_doubles);
  void release(void* p);
  // release for destructors and error paths: reports nothing
  void release_quiet(void* p) noexcept;
  void zero(double* p, int64_t n);

  // Slot table (slots other than X, Y, Combo and Ones).
  void set_slot(int slot, double* p);
  double* slot(int s) const { return host_slots_[s]; }
  // FP32 copy of a slot's buffer, read by FP32 runs (nullptr: none).
  void set_slot32(int slot, float* p);
  float* slot32(int s) const { return host_slots32_[s]; }
  float* alloc_f32(int64_t n_floats);

  std::unique_ptr<DevProgram> upload(const Program& p);
  // The program made of these shards (compiled with keep_empty from disjoint outputs), as
  // upload(merge_programs(parts)) gives it, without assembling the merged program.
  std::unique_ptr<DevProgram> upload(const std::vector<Program>& parts);
  void prepare(DevProgram& p);
  // Runs the repeat stages (preparing first if needed). The combination stage always runs
  // in FP64; prec selects the arithmetic of the repeat stages. An FP32 run converts X
  // (xlen elements) and the combined blocks to FP32 first and reads the FP32 slot copies
  // (set_slot32) of every other operand.
  void run(DevProgram& p, double* x, double* y, Precision prec = Precision::kFP64, int64_t xlen = 0);

  const double* ones(int64_t n);
  // Synchronises the runtime's streams, then throws if a kernel reported a failed bounded
  // wait since the last check (the device error word is cleared).
  void sync();
  void check_device_error();

  // Scratch for reductions and small Davidson quantities.
  double* partial() { return partial_; }
  // eight pinned host doubles for synchronising scalar reads on this stream (allocated with
  // the runtime: pinned allocations and frees synchronise the whole device)
  double* pinned_scalars() { return pinned_; }

 private:
  friend struct DevProgram;
  void flush_slots();
  SlotPtrs ptrs(double* x, double* y, double* combo);
  void launch_stage(const DevProgram& p, const DevStage& ds, const SlotPtrs& sp, Precision prec);
  enum TransientKind { kTransientInter, kTransientGemmPartials, kTransientGemmCounters, kTransientPartials,
                       kTransientCounters, kTransientKinds };
  void* transient_[kTransientKinds] = {};
  int64_t transient_cap_[kTransientKinds] = {};
  void* transient(int kind, int64_t bytes, bool zero);
  double* transient_doubles(int kind, int64_t n);
  unsigned int* transient_counters(int kind, int64_t n);

  int L_;
  int device_ = 0;
  cudaStream_t stream_ = nullptr;
  cudaStream_t aux_ = nullptr;
  cudaEvent_t fork_ev_ = nullptr, join_ev_ = nullptr;
  cudaEvent_t ext_in_ = nullptr, ext_out_ = nullptr;
  std::vector<double*> host_slots_;
  std::vector<float*> host_slots32_;
  const double** dev_slots_ = nullptr;
  const float** dev_slots32_ = nullptr;
  bool slots_dirty_ = true;
  float* x32_ = nullptr;  // FP32 copy of the X vector of an FP32 run
  int64_t x32_cap_ = 0;
  double* ones_ = nullptr;
  int64_t ones_cap_ = 0;
  double* partial_ = nullptr;
  double* pinned_ = nullptr;
  unsigned int* sched_ = nullptr;  // tile-scheduler counters of the tensor-core kernels
  int* err_host_ = nullptr;  // mapped pinned error word (host view)
  int* err_dev_ = nullptr;   // its device address
  // pinned host buffer in which upload assembles a program before the copy to the device
  // (the current one of a ring of two: a program is assembled in one while the copy of the
  // previous program from the other may still be in flight)
  char* staging_ = nullptr;
  int64_t staging_cap_ = 0;
  char* stg_buf_[2] = {nullptr, nullptr};
  int64_t stg_cap_[2] = {0, 0};
  cudaEvent_t stg_ev_[2] = {nullptr, nullptr};  // the copy out of each buffer
  bool stg_used_[2] = {false, false};
  int stg_next_ = 0;
  // program copies run here, so that an upload does not wait for the compute work queued
  // before it; the compute stream waits for each copy
  cudaStream_t copy_ = nullptr;
  // grows the staging buffer to at least `bytes`, keeping its first `keep` bytes
  void reserve_staging(int64_t bytes, int64_t keep);
  std::unique_ptr<DevProgram> upload_parts(const Program* parts, size_t np);
};

// Number of kernels this library has launched in this process (all runtimes).
int64_t kernel_launches();
void count_launches(int64_t n);

}  // namespace c2g

// A C++ caller of libqcu.so's reference-compatible operator interface
// (qcu_dirac.h, qcd/qcu_dslash.h): the three routes a reference user takes,
// on the reference's coalesced layouts.
//
//   dirac_caller DIR LX LY LZ LT NCOLORS NRHS PRECISION PARITY DAGGER
//
// DIR/gauge.bin  [4][2][N*N][Vh] complex (float2 for PRECISION 1, double2 for 2)
// DIR/in.bin     NRHS arrays [4N][Vh] complex, one parity each
// writes DIR/out_dirac.bin (qcu::DiracWilson::Dslash), DIR/out_inst.bin
// (qcu::instantiateDslash) and, for N = 3 and NRHS = 4, DIR/out_wd.bin
// (qcu::WilsonDslash<F, 3, 4>::apply); prints "errors <code>" after each call
// and after a call with an unsupported operator type.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "qcu_dirac.h"
#include "qcu_gb300.h"

static std::vector<char> read_file(const char* dir, const char* name) {
  char path[4096];
  snprintf(path, sizeof(path), "%s/%s", dir, name);
  FILE* f = fopen(path, "rb");
  if (!f) {
    fprintf(stderr, "cannot open %s\n", path);
    exit(2);
  }
  fseek(f, 0, SEEK_END);
  std::vector<char> b(ftell(f));
  fseek(f, 0, SEEK_SET);
  if (fread(b.data(), 1, b.size(), f) != b.size()) exit(2);
  fclose(f);
  return b;
}

static void write_file(const char* dir, const char* name, const std::vector<void*>& dev, size_t bytes) {
  char path[4096];
  snprintf(path, sizeof(path), "%s/%s", dir, name);
  FILE* f = fopen(path, "wb");
  std::vector<char> h(bytes);
  for (void* p : dev) {
    cudaMemcpy(h.data(), p, bytes, cudaMemcpyDeviceToHost);
    fwrite(h.data(), 1, bytes, f);
  }
  fclose(f);
}

int main(int argc, char** argv) {
  if (argc != 11) return 2;
  const char* dir = argv[1];
  const int L[4] = {atoi(argv[2]), atoi(argv[3]), atoi(argv[4]), atoi(argv[5])};
  const int N = atoi(argv[6]), nrhs = atoi(argv[7]), prec = atoi(argv[8]);
  const int parity = atoi(argv[9]), dagger = atoi(argv[10]);
  const size_t vh = (size_t)L[0] * L[1] * L[2] * L[3] / 2;
  const size_t cbytes = prec == 2 ? 16 : 8;
  const size_t fbytes = vh * 4 * N * cbytes;
  std::vector<char> hg = read_file(dir, "gauge.bin"), hin = read_file(dir, "in.bin");
  void* gauge = nullptr;
  cudaMalloc(&gauge, hg.size());
  cudaMemcpy(gauge, hg.data(), hg.size(), cudaMemcpyHostToDevice);
  std::vector<void*> in(nrhs), out(nrhs);
  for (int r = 0; r < nrhs; r++) {
    cudaMalloc(&in[r], fbytes);
    cudaMalloc(&out[r], fbytes);
    cudaMemcpy(in[r], hin.data() + r * fbytes, fbytes, cudaMemcpyHostToDevice);
  }
  const QCU_PRECISION fp = prec == 2 ? QCU_DOUBLE_PRECISION : QCU_SINGLE_PRECISION;
  QcuLattDesc<Nd> latt(L[0], L[1], L[2], L[3]);
  QcuProcDesc<Nd> proc(1, 1, 1, 1);
  qcu::ExecutionStreams streams;

  qcu::DiracWilson dirac(gauge, 0.1, N, fp, latt, proc, DSLASH_WILSON, streams);
  qcu::Dirac* op = &dirac;  // through the base class, as the reference's users hold it
  op->Dslash(out.data(), in.data(), parity, dagger, nrhs);
  printf("errors %d\n", qcuGetLastError());
  write_file(dir, "out_dirac.bin", out, fbytes);

  for (void* p : out) cudaMemset(p, 0, fbytes);
  qcu::instantiateDslash(latt, proc, parity, dagger, 0.12, in.data(), out.data(), gauge, DSLASH_WILSON, fp, N, nrhs,
                         streams);
  printf("errors %d\n", qcuGetLastError());
  write_file(dir, "out_inst.bin", out, fbytes);

  if (N == 3 && nrhs == 4) {
    for (void* p : out) cudaMemset(p, 0, fbytes);
    qcu::MrhsInput<4> mi, mo;
    for (int r = 0; r < 4; r++) mi.fermion[r] = in[r], mo.fermion[r] = out[r];
    qcu::DslashParam param(latt, proc, parity, dagger, 0.12, &mi, &mo, gauge, streams);
    if (prec == 2) {
      qcu::WilsonDslash<double, 3, 4> wd(param);
      wd.preApply();
      wd.apply();
      wd.postApply();
    } else {
      qcu::WilsonDslash<float, 3, 4> wd(param);
      wd.preApply();
      wd.apply();
      wd.postApply();
    }
    printf("errors %d\n", qcuGetLastError());
    write_file(dir, "out_wd.bin", out, fbytes);
  }
  // an operator type the library does not implement: reported, not fatal
  qcu::instantiateDslash(latt, proc, parity, dagger, 0.12, in.data(), out.data(), gauge, DSLASH_CLOVER, fp, N, nrhs,
                         streams);
  printf("errors %d\n", qcuGetLastError());
  qcuClearError();
  return 0;
}

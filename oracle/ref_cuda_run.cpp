// ref_cuda_run.cpp -- TEST INFRASTRUCTURE ONLY: runs kernels of the reference's own
// CUDA code on a GPU to produce fixtures for the CUDA-only parts of the path.
//
// The two-point contact rule, the pure-shear step and the conjugate-gradient
// primitives exist only in tmarschall/spherocyls' src/cuda.  oracle/Makefile
// (target ref_cuda) compiles src/cuda/2point_dynamics.cu where it lies into a
// device-code module (oracle/_ref/ref2p.cubin); this program, compiled on the GPU
// machine, loads that module with the CUDA driver API, finds the kernels by name
// and launches them on the inputs of one case.  The host code around the kernels
// is the reference's host sequence restated: one pure-shear step is
// pure_euler_est_2p, pure_heun_corr_2p at the half-step box, then the box update
// (Spherocyl_Box::pure_strain_step_2p, src/cuda/2point_dynamics.cu:2180-2283).
//
//   ref_cuda_run <module.cubin> <case.bin> <out.bin>
//
// case.bin (little endian): int32 mode (1: forces and energy, calc_fe_2p; 2: one
// pure-shear step), int32 n, int32 max_nbrs; float64 Lx, Ly, gamma, strain rate,
// step, epsilon (the list padding), kd; float64 x, y, phi, R, A, area, moi, isoc
// [n each]; int32 nnbr [n]; int32 nbr [max_nbrs * n] (column-major, entry k of
// particle i at k * n + i).
// out.bin: mode 1: float64 fx, fy, tau [n each], energy (the sum of the block
// energies); mode 2: float64 x, y, phi, fx, fy, tau [n each], Lx, Ly, int32 new_nbrs.
#include <cuda.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

void check(CUresult r, const char* what) {
  if (r != CUDA_SUCCESS) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    std::fprintf(stderr, "ref_cuda_run: %s: %s\n", what, s ? s : "?");
    std::exit(2);
  }
}

// the kernel whose mangled name contains `key` (an instantiation of a template)
CUfunction find_kernel(CUmodule mod, const char* key) {
  unsigned count = 0;
  check(cuModuleGetFunctionCount(&count, mod), "function count");
  std::vector<CUfunction> fs(count);
  check(cuModuleEnumerateFunctions(fs.data(), count, mod), "enumerate functions");
  for (CUfunction f : fs) {
    const char* name = nullptr;
    if (cuFuncGetName(&name, f) == CUDA_SUCCESS && name && std::strstr(name, key)) return f;
  }
  std::fprintf(stderr, "ref_cuda_run: no kernel matching %s\n", key);
  std::exit(2);
}

struct Reader {
  FILE* f;
  template <class T>
  std::vector<T> get(size_t n) {
    std::vector<T> v(n);
    if (n && std::fread(v.data(), sizeof(T), n, f) != n) {
      std::fprintf(stderr, "ref_cuda_run: short input\n");
      std::exit(2);
    }
    return v;
  }
};

template <class T>
CUdeviceptr upload(const std::vector<T>& v) {
  CUdeviceptr p = 0;
  check(cuMemAlloc(&p, v.size() * sizeof(T) + 16), "alloc");
  if (!v.empty()) check(cuMemcpyHtoD(p, v.data(), v.size() * sizeof(T)), "upload");
  return p;
}

template <class T>
std::vector<T> download(CUdeviceptr p, size_t n) {
  std::vector<T> v(n);
  if (n) check(cuMemcpyDtoH(v.data(), p, n * sizeof(T)), "download");
  return v;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: ref_cuda_run <module.cubin> <case.bin> <out.bin>\n");
    return 1;
  }
  FILE* in = std::fopen(argv[2], "rb");
  if (!in) {
    std::perror(argv[2]);
    return 1;
  }
  Reader rd{in};
  const auto head = rd.get<int>(3);
  const int mode = head[0], n = head[1], maxn = head[2];
  if ((mode != 1 && mode != 2) || n < 1 || maxn < 1) {
    std::fprintf(stderr, "ref_cuda_run: bad header\n");
    return 1;
  }
  const auto sc = rd.get<double>(7);
  double Lx = sc[0], Ly = sc[1];
  const double gamma = sc[2], rate = sc[3], step = sc[4], eps = sc[5], kd = sc[6];
  auto x = rd.get<double>(n), y = rd.get<double>(n), phi = rd.get<double>(n);
  const auto R = rd.get<double>(n), A = rd.get<double>(n), area = rd.get<double>(n);
  const auto moi = rd.get<double>(n), isoc = rd.get<double>(n);
  const auto nnbr = rd.get<int>(n);
  const auto nbr = rd.get<int>((size_t)maxn * n);
  std::fclose(in);
  for (int i = 0; i < n; i++)
    for (int k = 0; k < nnbr[i]; k++) {
      const int j = nbr[(size_t)k * n + i];
      if (nnbr[i] > maxn || j < 0 || j >= n) {
        std::fprintf(stderr, "ref_cuda_run: neighbour list out of range\n");
        return 1;
      }
    }

  check(cuInit(0), "init");
  CUdevice dev;
  check(cuDeviceGet(&dev, 0), "device");
  CUcontext ctx;
  check(cuDevicePrimaryCtxRetain(&ctx, dev), "context");
  check(cuCtxSetCurrent(ctx), "context");
  CUmodule mod;
  check(cuModuleLoad(&mod, argv[1]), "module load");

  CUdeviceptr dnn = upload(nnbr), dnb = upload(nbr);
  CUdeviceptr dx = upload(x), dy = upload(y), dp = upload(phi), dR = upload(R), dA = upload(A);
  CUdeviceptr darea = upload(area), dmoi = upload(moi), diso = upload(isoc);
  const std::vector<double> zero(n, 0.0);
  CUdeviceptr dfx = upload(zero), dfy = upload(zero), dft = upload(zero);
  const int block = 256, grid = (n + block - 1) / block;
  FILE* out = std::fopen(argv[3], "wb");
  if (!out) {
    std::perror(argv[3]);
    return 1;
  }
  if (mode == 1) {
    // calc_fe_2p<HARMONIC> (src/cuda/2point_dynamics.cu:2714-2962): forces, torques
    // and per-block energies; the reference launches it with blockDim doubles of
    // shared memory (:3798)
    CUfunction fe = find_kernel(mod, "calc_fe_2pIL9Potential2E");
    CUdeviceptr deb = upload(std::vector<double>(grid, 0.0));
    int nn = n;
    void* args[] = {&nn, &dnn, &dnb, &Lx, &Ly, (void*)&gamma, &dx, &dy, &dp, &dR, &dA,
                    &dmoi, &dfx, &dfy, &dft, &deb};
    check(cuLaunchKernel(fe, grid, 1, 1, block, 1, 1, block * sizeof(double), nullptr, args,
                         nullptr), "calc_fe_2p");
    check(cuCtxSynchronize(), "calc_fe_2p sync");
    const auto fx = download<double>(dfx, n), fy = download<double>(dfy, n);
    const auto ft = download<double>(dft, n), eb = download<double>(deb, grid);
    double e = 0.0;
    for (double v : eb) e += v;
    std::fwrite(fx.data(), sizeof(double), n, out);
    std::fwrite(fy.data(), sizeof(double), n, out);
    std::fwrite(ft.data(), sizeof(double), n, out);
    std::fwrite(&e, sizeof(double), 1, out);
  } else {
    // pure_strain_step_2p without stress (src/cuda/2point_dynamics.cu:2180-2283)
    CUfunction est = find_kernel(mod, "pure_euler_est_2pIL9Potential2ELi0E");
    CUfunction corr = find_kernel(mod, "pure_heun_corr_2pIL9Potential2E");
    CUdeviceptr dtx = upload(zero), dty = upload(zero), dtp = upload(zero);
    CUdeviceptr dxm = upload(zero), dym = upload(zero);
    CUdeviceptr dnew = upload(std::vector<int>(1, 0));
    CUdeviceptr dse = upload(std::vector<float>(5, 0.f));
    int nn = n;
    double kdv = kd, g = gamma, r = rate, st = step, ep = eps;
    void* a1[] = {&nn, &dnn, &dnb, &Lx, &Ly, &g, &r, &st, &dx, &dy, &dp, &dR, &dA, &kdv,
                  &darea, &dmoi, &diso, &dfx, &dfy, &dft, &dse, &dtx, &dty, &dtp};
    check(cuLaunchKernel(est, grid, 1, 1, block, 1, 1, 0, nullptr, a1, nullptr),
          "pure_euler_est_2p");
    check(cuCtxSynchronize(), "pure_euler_est_2p sync");
    double Lxh = Lx * (1 + 0.5 * step * rate), Lyh = Ly * (1 - 0.5 * step * rate);
    void* a2[] = {&nn, &dnn, &dnb, &Lxh, &Lyh, &g, &r, &st, &dx, &dy, &dp, &dR, &dA, &kdv,
                  &darea, &dmoi, &diso, &dfx, &dfy, &dft, &dtx, &dty, &dtp, &dxm, &dym, &ep,
                  &dnew};
    check(cuLaunchKernel(corr, grid, 1, 1, block, 1, 1, 0, nullptr, a2, nullptr),
          "pure_heun_corr_2p");
    check(cuCtxSynchronize(), "pure_heun_corr_2p sync");
    Lx += 0.5 * step * rate * Lx;
    Ly -= 0.5 * step * rate * Ly;
    x = download<double>(dx, n);
    y = download<double>(dy, n);
    phi = download<double>(dp, n);
    const auto fx = download<double>(dfx, n), fy = download<double>(dfy, n);
    const auto ft = download<double>(dft, n);
    const auto nw = download<int>(dnew, 1);
    const std::vector<double>* outs[] = {&x, &y, &phi, &fx, &fy, &ft};
    for (const auto* v : outs) std::fwrite(v->data(), sizeof(double), n, out);
    std::fwrite(&Lx, sizeof(double), 1, out);
    std::fwrite(&Ly, sizeof(double), 1, out);
    std::fwrite(nw.data(), sizeof(int), 1, out);
  }
  std::fclose(out);
  check(cuModuleUnload(mod), "unload");
  check(cuDevicePrimaryCtxRelease(dev), "release");
  return 0;
}

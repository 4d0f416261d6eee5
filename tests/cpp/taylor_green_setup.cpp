// A setup written against the reference's LBM interface (the pattern of src/setup.cpp:40-59 and its
// "binary identity" probe at :58), compiled against fluidx3d_gb300/host/lbm.hpp: 64^3 Taylor-Green
// vortex, D3Q19 SRT FP32, nu = 1/30, 1000 steps. Writes rho and u (raw float32) to argv[1] and
// prints u.x at the box centre.
#define EXACT_ARITHMETIC // bit-identical to the reference
#include "lbm.hpp"

int main(int argc, char** argv) {
	if(argc<2) { std::fprintf(stderr, "usage: %s out.bin\n", argv[0]); return 2; }
	LBM lbm(64u, 64u, 64u, 1.0f/30.0f);
	const uint Nx = lbm.get_Nx(), Ny = lbm.get_Ny(), Nz = lbm.get_Nz();
	FILE* init = std::fopen(argv[1], "rb"); // initial rho/u written by the test (the same seeded arrays the oracle uses)
	if(!init) { std::fprintf(stderr, "missing initial state\n"); return 2; }
	const ulong N = lbm.get_N();
	if(std::fread(lbm.rho.host(), 4, N, init)!=N || std::fread(lbm.u.host(), 4, 3u*N, init)!=3u*N) return 2;
	std::fclose(init);
	lbm.run(1000u);
	lbm.rho.read_from_device();
	lbm.u.read_from_device();
	std::printf("ux_center %.9g t %llu\n", lbm.u.x[lbm.index(Nx/2u, Ny/2u, Nz/2u)], (unsigned long long)lbm.get_t());
	FILE* out = std::fopen(argv[1], "wb");
	std::fwrite(lbm.rho.host(), 4, N, out);
	std::fwrite(lbm.u.host(), 4, 3u*N, out);
	std::fclose(out);
	return 0;
}

// VTK export and STL import through the C++ host layer (fluidx3d_gb300/host/lbm.hpp), as a setup of
// the reference would use them (src/lbm.hpp:298-340, 401-407; src/lbm.cpp:1094-1129;
// src/utilities.hpp:4530-4581). Compile with -DVOLUME_FORCE -DFORCE_FIELD -DEQUILIBRIUM_BOUNDARIES.
//   vtk_export_setup <out folder> <binary STL file>
// writes <out>/device/{rho,u,flags,F}-000000010.vtk straight from the GPU, the same from the host
// copies into <out>/host/, <out>/si/ with SI units, and <out>/mesh-000000010.vtk from the STL.
#include <cstdio>
#include "lbm.hpp"

int main(int argc, char** argv) {
	if(argc<3) { std::fprintf(stderr, "usage: %s <out folder> <stl file>\n", argv[0]); return 2; }
	const std::string out = std::string(argv[1])+"/", stl = argv[2];
	LBM lbm(40u, 24u, 20u, 0.05f, 1e-5f, 0.0f, 0.0f);
	const uint Nx = lbm.get_Nx(), Ny = lbm.get_Ny(), Nz = lbm.get_Nz();
	for(ulong n=0ull; n<lbm.get_N(); n++) {
		uint x = 0u, y = 0u, z = 0u;
		lbm.coordinates(n, x, y, z);
		const float dx = (float)x-12.0f, dy = (float)y-11.5f, dz = (float)z-9.5f;
		if(dx*dx+dy*dy+dz*dz<=25.0f) lbm.flags[n] = TYPE_S|TYPE_X;
		else if(y==0u||y==Ny-1u||z==0u||z==Nz-1u) lbm.flags[n] = TYPE_S;
		else if(x==0u||x==Nx-1u) lbm.flags[n] = TYPE_E;
		if(lbm.flags[n]!=TYPE_S && lbm.flags[n]!=(TYPE_S|TYPE_X)) lbm.u.x[n] = 0.05f;
	}
	lbm.run(10u);
	lbm.update_force_field();
	lbm.rho.write_device_to_vtk(out+"device/", false);
	lbm.u.write_device_to_vtk(out+"device/", false);
	lbm.flags.write_device_to_vtk(out+"device/", false);
	lbm.F.write_device_to_vtk(out+"device/", false);
	lbm.rho.read_from_device(); lbm.u.read_from_device(); lbm.flags.read_from_device(); lbm.F.read_from_device();
	lbm.rho.write_host_to_vtk(out+"host/", false);
	lbm.u.write_host_to_vtk(out+"host/", false);
	lbm.flags.write_host_to_vtk(out+"host/", false);
	lbm.F.write_host_to_vtk(out+"host/", false);
	units.set_m_kg_s(38.0f, 0.05f, 1.0f, 0.2f, 1.5f, 1000.0f); // 38 cells = 0.2 m, u 0.05 = 1.5 m/s, water
	lbm.u.write_device_to_vtk(out+"si/device/");
	lbm.u.write_host_to_vtk(out+"si/host/");
	lbm.F.write_device_to_vtk(out+"si/device/");
	lbm.F.write_host_to_vtk(out+"si/host/");
	Mesh* mesh = read_stl(stl, lbm.size(), lbm.center(), float3x3(0.0f, -1.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f), 16.0f);
	lbm.write_mesh_to_vtk(mesh, out, false);
	std::printf("t %llu triangles %u pmin %.9g %.9g %.9g pmax %.9g %.9g %.9g si %.9g %.9g %.9g\n", (unsigned long long)lbm.get_t(), mesh->triangle_number,
	            mesh->pmin.x, mesh->pmin.y, mesh->pmin.z, mesh->pmax.x, mesh->pmax.y, mesh->pmax.z, units.si_x(1.0f), units.si_u(1.0f), units.si_F(1.0f));
	delete mesh;
	return 0;
}

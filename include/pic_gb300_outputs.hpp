// pic_gb300_outputs.hpp -- the reference's output writers (ch4/v3/src/Outputs.{h,cpp}) over the
// C++ facade: ASCII VTK ImageData fields, VTK PolyData particle samples, runtime_diags.csv,
// the screen line and convergence.csv.  The files, array names, column names and number
// layout are those of the reference, so its ParaView states and analysis scripts read them
// unchanged.  Fields are staged from the device through the C ABI once per call.
//
// The species list may hold Species objects or pointers to them.
#ifndef PIC_GB300_OUTPUTS_HPP
#define PIC_GB300_OUTPUTS_HPP
#include <algorithm>
#include <cctype>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
#include "pic_gb300.hpp"

namespace pic_gb300 {
namespace Output {

enum modes { none, all, screen, fields, particles, diagnostics, convergence };  // Outputs.h:12

namespace detail {
// Field<T> << : per z plane, x fastest, "v " each and a newline after the plane (Field.h:676-692)
template <class T>
void write_scalar(std::ostream& out, const std::vector<T>& a, size_t plane) {
    for (size_t n = 0; n < a.size(); n++) {
        out << a[n] << " ";
        if ((n + 1) % plane == 0) out << "\n";
    }
}
// Field<Vec3> << : each node as Vec3 << (Vec3.h:372-375) then " "
inline void write_vec3(std::ostream& out, const std::vector<double>& a, size_t plane) {
    const size_t nv = a.size() / 3;
    for (size_t n = 0; n < nv; n++) {
        out << std::setw(5) << a[3 * n] << " " << std::setw(5) << a[3 * n + 1] << " " << std::setw(5) << a[3 * n + 2]
            << " ";
        if ((n + 1) % plane == 0) out << "\n";
    }
}
inline void array_head(std::ostream& out, const std::string& name, int comps) {
    out << "<DataArray Name=\"" << name << "\" NumberOfComponents=\"" << comps << "\" format=\"ascii\" type=\"Float64\">\n";
}
inline std::string ts5(int ts) {
    std::stringstream s;
    s << std::setfill('0') << std::setw(5) << ts;
    return s.str();
}
inline std::ofstream& f_diag() {
    static std::ofstream f;
    return f;
}
inline std::ofstream& f_convergence() {
    static std::ofstream f;
    return f;
}
}  // namespace detail

// results/<name1>fields_<ts>.vti (Outputs.cpp:9-123); clears the velocity samples afterwards
// unless the world has reached a steady state
template <class V>
void fieldsOutput(World& world, V& species, std::string name1 = "") {
    for (auto& x : species) pic_gb300::detail::sp_ref(x).computeGasProperties();
    std::string name = "results/" + name1 + "fields_" + detail::ts5(world.getTs()) + ".vti";
    std::ofstream out(name);
    if (!out.is_open()) {
        std::cerr << "Could not open " << name << std::endl;
        return;
    }
    const size_t plane = (size_t)world.ni * world.nj, cplane = (size_t)(world.ni - 1) * (world.nj - 1);
    type_calc3 x0 = world.getX0(), dx = world.getDx();
    out << "<VTKFile type=\"ImageData\">\n";
    out << "<ImageData Origin=\"" << x0[0] << " " << x0[1] << " " << x0[2] << "\" ";
    out << "Spacing=\"" << dx[0] << " " << dx[1] << " " << dx[2] << "\" ";
    out << "WholeExtent=\"0 " << world.ni - 1 << " 0 " << world.nj - 1 << " 0 " << world.nk - 1 << "\">\n";
    out << "<PointData>\n";
    auto scalar = [&](const std::string& n, const std::vector<double>& a) {
        detail::array_head(out, n, 1);
        detail::write_scalar(out, a, plane);
        out << "</DataArray>\n";
    };
    auto as_int = [](const std::vector<double>& a) {
        std::vector<int> r(a.size());
        for (size_t n = 0; n < a.size(); n++) r[n] = (int)a[n];
        return r;
    };
    scalar("NodeVol", world.node_vol());
    {
        detail::array_head(out, "ObjectID", 1);
        detail::write_scalar(out, as_int(world.object_id()), plane);
        out << "</DataArray>\n";
        detail::array_head(out, "NodeType", 1);
        detail::write_scalar(out, as_int(world.node_type()), plane);
        out << "</DataArray>\n";
    }
    scalar("phi", world.phi());
    scalar("rho", world.rho());
    for (auto& x : species) {
        Species& sp = pic_gb300::detail::sp_ref(x);
        scalar("nd." + sp.name, sp.den());
    }
    for (auto& x : species) {
        Species& sp = pic_gb300::detail::sp_ref(x);
        scalar("avg_nd." + sp.name, sp.den_avg());
    }
    for (auto& x : species) {
        Species& sp = pic_gb300::detail::sp_ref(x);
        detail::array_head(out, "vel." + sp.name, 3);
        detail::write_vec3(out, sp.vel, plane);
        out << "</DataArray>\n";
    }
    for (auto& x : species) {
        Species& sp = pic_gb300::detail::sp_ref(x);
        scalar("T." + sp.name, sp.T);
    }
    detail::array_head(out, "ef", 3);
    detail::write_vec3(out, world.ef(), plane);
    out << "</DataArray>\n";
    out << "</PointData>\n";
    out << "<CellData>\n";
    for (auto& x : species) {
        Species& sp = pic_gb300::detail::sp_ref(x);
        std::vector<int32_t> mpc = sp.macro_part_count;
        mpc.resize((size_t)world.num_cells, 0);  // zero until computeMacroParticlesCount ran
        detail::array_head(out, "mpc." + sp.name, 1);
        detail::write_scalar(out, mpc, cplane);
        out << "</DataArray>\n";
    }
    out << "</CellData>\n";
    out << "</ImageData>\n";
    out << "</VTKFile>\n";
    out.close();
    if (!world.steadyState())
        for (auto& x : species) pic_gb300::detail::sp_ref(x).clearSamples();
}

// the progress line (Outputs.cpp:127-135)
template <class V>
void screenOutput(World& world, V& species) {
    std::cout << "\r                                                                  \rts: " << world.getTs();
    for (auto& x : species) {
        Species& sp = pic_gb300::detail::sp_ref(x);
        std::cout << std::setprecision(3) << "\t " << sp.name << ":" << sp.getNumParticles() << " ";
    }
    std::cout << std::flush;
}

// one row of results/runtime_diags.csv (Outputs.cpp:143-182); the header on the first call
template <class V>
void diagOutput(World& world, V& species) {
    std::ofstream& f = detail::f_diag();
    if (!f.is_open()) {
        f.open("results/runtime_diags.csv");
        f << "ts,time,wall_time";
        for (auto& x : species) {
            const std::string& n = pic_gb300::detail::sp_ref(x).name;
            f << ",mp_count." << n << ",real_count." << n << ",px." << n << ",py." << n << ",pz." << n << ",KE." << n;
        }
        f << ",PE,E_total" << std::endl;
    }
    f << world.getTs() << "," << world.getTime();
    f << "," << world.getWallTime();
    double tot_KE = 0;
    for (auto& x : species) {
        Species& sp = pic_gb300::detail::sp_ref(x);
        double KE = sp.getKE();
        tot_KE += KE;
        type_calc3 mom = sp.getMomentum();
        f << "," << sp.getNumParticles() << "," << sp.getMicroCount() << "," << mom[0] << "," << mom[1] << ","
          << mom[2] << "," << KE;
    }
    double PE = world.getPE();
    f << "," << PE << "," << (tot_KE + PE);
    f << "\n";
    if (world.getTs() % 25 == 0) f.flush();
}
// closes runtime_diags.csv (the reference leaves it to program exit)
inline void closeDiagOutput() {
    if (detail::f_diag().is_open()) detail::f_diag().close();
}

// convergence.csv rows (Outputs.cpp:185-204)
inline void convergenceOutput(type_calc L2, int it, int ts) {
    std::ofstream& f = detail::f_convergence();
    if (!f.is_open()) {
        f.open("convergence.csv");
        f << "L2,PCG_it,ts,NR_it\n";
    }
    f << L2 << "," << it << "," << ts << ",\n";
}
inline void convergenceOutput(int NR_it, int ts) {
    std::ofstream& f = detail::f_convergence();
    if (!f.is_open()) {
        f.open("convergence.csv");
        f << "L2,PCG_it,ts,NR_it\n";
    }
    f << "," << "," << ts << "," << NR_it << "\n";
}

// results/<name1>parts_<species>_<ts>.vtp per species: num_parts_to_output_base particles
// picked as in the reference (every n / num-th, Outputs.cpp:207-290)
template <class V>
void particlesOutput(World& world, V& species, int num_parts_to_output_base, std::string name1 = "") {
    for (auto& x : species) {
        Species& sp = pic_gb300::detail::sp_ref(x);
        std::string name = "results/" + name1 + "parts_" + sp.name + "_" + detail::ts5(world.getTs()) + ".vtp";
        std::ofstream out(name);
        if (!out.is_open()) {
            std::cerr << "Could not open " << name << std::endl;
            return;
        }
        std::vector<Particle> to_output;
        if (sp.getNumParticles() != 0) to_output = sp.sampleParticles(num_parts_to_output_base);
        out << "<?xml version=\"1.0\"?>\n";
        out << "<VTKFile type=\"PolyData\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
        out << "<PolyData>\n";
        out << "<Piece NumberOfPoints=\"" << to_output.size() << "\" NumberOfVerts=\"0\" NumberOfLines=\"0\" ";
        out << "NumberOfStrips=\"0\" NumberOfCells=\"0\">\n";
        out << "<Points>\n";
        out << "<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n";
        for (const Particle& p : to_output)
            out << std::setw(5) << p.pos[0] << " " << std::setw(5) << p.pos[1] << " " << std::setw(5) << p.pos[2] << "\n";
        out << "</DataArray>\n";
        out << "</Points>\n";
        out << "<PointData>\n";
        out << "<DataArray Name=\"vel." << sp.name << "\" type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n";
        for (const Particle& p : to_output)
            out << std::setw(5) << p.vel[0] << " " << std::setw(5) << p.vel[1] << " " << std::setw(5) << p.vel[2] << "\n";
        out << "</DataArray>\n";
        out << "</PointData>\n";
        out << "</Piece>\n";
        out << "</PolyData>\n";
        out << "</VTKFile>\n";
        out.close();
    }
}

// --output names and numbers (Outputs.cpp:293-383); an unknown value falls back to fields
inline std::istream& operator>>(std::istream& in, modes& type) {
    std::string input;
    in >> input;
    std::transform(input.begin(), input.end(), input.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    if (input == "none" || input == "0") type = none;
    else if (input == "all" || input == "1") type = all;
    else if (input == "screen" || input == "2") type = screen;
    else if (input == "fields" || input == "3") type = fields;
    else if (input == "particles" || input == "4") type = particles;
    else if (input == "diagnostics" || input == "5") type = diagnostics;
    else if (input == "convergence" || input == "6") type = convergence;
    else {
        std::cerr << "Wrong Output::modes value, setting Output::modes::fields \n";
        type = fields;
    }
    return in;
}
inline std::ostream& operator<<(std::ostream& out, const modes& type) {
    static const char* names[] = {"none", "all", "screen", "fields", "particles", "diagnostics", "convergence"};
    if (type >= none && type <= convergence) out << names[type];
    return out;
}

}  // namespace Output
}  // namespace pic_gb300
#endif

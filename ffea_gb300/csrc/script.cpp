// script.cpp -- the .ffea script front end: FFEA's input script and blob
// files read into the arrays ffea_gpu_create_batch takes.
//
// The script language is FFEA's (src/FFEA_input_reader.cpp,
// src/SimulationParams.cpp:184-550, src/World.cpp:2205-2720): lines of
// <key = value> tags in <param> and <system><blob><conformation> blocks,
// <!-- --> comments, file names relative to the script's directory.  The
// units are converted as SimulationParams::assign and Blob::init convert
// them.  The blob files (.node, .top, .mat, .stokes, .pin) are read as
// Blob::load_nodes / load_topology / load_material_params /
// load_stokes_params / load_pinned_nodes read them (src/Blob.cpp:2415-2947,
// 3691-3755).
//
// Supported: the parameters of the blob update (dt, kT, epsilon,
// max_iterations_cg, calc_noise, calc_stokes / do_stokes, stokes_visc,
// rng_seed), the run control (num_steps, check, restart, output and
// checkpoint names), and per blob one DYNAMIC conformation with nodes,
// topology, material, stokes and pin files, solver CG_nomass / CG /
// masslumped, scale, centroid and velocity.  Every other parameter FFEA
// knows is accepted and recorded as read; those that switch on work outside
// the blob update (surface-surface interactions, electrostatics, kinetics,
// springs, constant forces, precomputed potentials, rods) are rejected, as
// are several conformations, STATIC / FROZEN blobs, rotations and the direct
// solver.  calc_steric is accepted but not computed here (steric repulsion
// acts only between overlapping faces).
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ffea_gpu.h"

namespace ffea {
void set_last_error(const char *msg);  // api.cu
}

namespace {

// include/dimensions.h:30-41
constexpr double kMesoLength = 1.7e-10;
constexpr double kMesoEnergy = 4.141945559999999e-21;
constexpr double kMesoMass = 1.994307387553024e-26;
constexpr double kMesoVolume = 4.913e-30;
constexpr double kMesoTime = 3.7302915560886126e-13;
constexpr double kMesoPressure = 8.4305832688784826e8;
constexpr double kMesoVelocity = 4.5572845297447225e2;
constexpr double kPi = 3.14159265358979323846264338327950288;  // include/mat_vec_types.h:54

struct Error {
    std::string msg;
};

[[noreturn]] void raise(const std::string &m) { throw Error{m}; }

std::string trim(const std::string &s)
{
    const char *ws = " \t\r\n";
    const size_t a = s.find_first_not_of(ws);
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(ws);
    return s.substr(a, b - a + 1);
}

// FFEA_input_reader::file_to_lines: comments <!-- --> removed (they may span
// lines), each line trimmed, empty lines dropped.
std::vector<std::string> script_lines(const std::string &path)
{
    std::ifstream in(path);
    if (!in) raise(path + " does not exist");
    std::vector<std::string> out;
    std::string line;
    bool comment = false;
    while (std::getline(in, line)) {
        std::string kept;
        size_t i = 0;
        while (i <= line.size()) {
            if (comment) {
                const size_t e = line.find("-->", i);
                if (e == std::string::npos) break;
                comment = false;
                i = e + 3;
            } else {
                const size_t b = line.find("<!--", i);
                if (b == std::string::npos) {
                    kept += line.substr(i);
                    break;
                }
                kept += line.substr(i, b - i);
                comment = true;
                i = b + 4;
            }
        }
        kept = trim(kept);
        if (!kept.empty()) out.push_back(kept);
    }
    return out;
}

// The tag name of a line: "<name ...>" -> "name" (FFEA_input_reader::extract_block)
std::string tag_name(const std::string &line)
{
    std::string s = line;
    if (!s.empty() && s.front() == '<') s.erase(0, 1);
    if (!s.empty() && s.back() == '>') s.pop_back();
    s = trim(s);
    const size_t sp = s.find(' ');
    return sp == std::string::npos ? s : s.substr(0, sp);
}

// Lines strictly inside the index-th <title> ... </title> block; false when
// there is no such block.
bool extract_block(const std::vector<std::string> &in, const std::string &title, int index,
                   std::vector<std::string> &out)
{
    out.clear();
    int count = -1;
    bool copying = false;
    for (const std::string &l : in) {
        const std::string t = tag_name(l);
        if (t == title) {
            if (copying) raise("found '" + title + "' inside a '" + title + "' block");
            if (++count == index) {
                copying = true;
                continue;
            }
        }
        if (copying) {
            if (t == "/" + title) return true;
            out.push_back(l);
        }
    }
    if (copying) raise("never found the closing tag '/" + title + "'");
    return false;
}

// "<key = value>" -> key, value (FFEA_input_reader::parse_tag)
void parse_tag(const std::string &line, std::string &key, std::string &value)
{
    if (line.find('<') == std::string::npos) raise("line '" + line + "' is missing '<'");
    if (line.find('>') == std::string::npos) raise("line '" + line + "' is missing '>'");
    std::string s = line.substr(line.find('<') + 1);
    s = s.substr(0, s.rfind('>'));
    const size_t eq = s.find('=');
    key = trim(eq == std::string::npos ? s : s.substr(0, eq));
    value = eq == std::string::npos ? "" : trim(s.substr(eq + 1));
}

double to_double(const std::string &v, const std::string &key)
{
    errno = 0;
    char *end = nullptr;
    const double x = std::strtod(v.c_str(), &end);
    if (end == v.c_str() || errno == ERANGE) raise("parameter " + key + " = '" + v + "' is not a number");
    return x;
}

// atoi / (long long)atof as SimulationParams::assign reads integers
int to_int(const std::string &v, const std::string &key)
{
    (void)key;
    return std::atoi(v.c_str());
}

// "(a, b, c)" -> numbers
std::vector<double> to_list(std::string v, const std::string &key)
{
    v = trim(v);
    if (!v.empty() && v.front() == '(') v.erase(0, 1);
    if (!v.empty() && v.back() == ')') v.pop_back();
    std::vector<double> out;
    std::stringstream ss(v);
    std::string item;
    while (std::getline(ss, item, ',')) out.push_back(to_double(trim(item), key));
    return out;
}

std::string join(const std::string &dir, const std::string &name)
{
    if (name.empty() || name[0] == '/' || dir.empty()) return name;
    return dir + "/" + name;
}

void copy_name(char *dst, const std::string &s)
{
    if (s.size() >= FFEA_GPU_SCRIPT_PATH_MAX) raise("file name longer than the supported maximum: " + s);
    std::strncpy(dst, s.c_str(), FFEA_GPU_SCRIPT_PATH_MAX - 1);
    dst[FFEA_GPU_SCRIPT_PATH_MAX - 1] = '\0';
}

// ---- blob files ---------------------------------------------------------

struct Lines {
    std::vector<std::string> v;
    std::string path;
    explicit Lines(const std::string &p) : path(p)
    {
        std::ifstream in(p);
        if (!in) raise(p + " does not exist");
        std::string l;
        while (std::getline(in, l)) v.push_back(l);
    }
    const std::string &at(size_t i) const
    {
        if (i >= v.size()) raise(path + ": unexpected end of file");
        return v[i];
    }
    void magic(const char *a, const char *b) const
    {
        const std::string m = trim(at(0));
        if (m != a && m != b) raise(path + ": not an FFEA '" + a + "'");
    }
    long header(size_t i, const char *key) const
    {
        std::stringstream ss(at(i));
        std::string k;
        long n = -1;
        ss >> k >> n;
        if (k != key || n < 0) raise(path + ": expected '" + key + " <n>' at line " + std::to_string(i + 1));
        return n;
    }
    void expect(size_t i, const char *text) const
    {
        if (trim(at(i)) != text) raise(path + ": expected '" + text + "' at line " + std::to_string(i + 1));
    }
};

std::vector<double> numbers(const Lines &L, size_t i, int want)
{
    std::stringstream ss(L.at(i));
    std::vector<double> out;
    std::string tok;
    while ((int)out.size() < want && ss >> tok) out.push_back(to_double(tok, L.path));
    if ((int)out.size() < want) raise(L.path + ": too few values at line " + std::to_string(i + 1));
    return out;
}

// Blob::load_nodes: header, surface nodes, interior nodes (x y z each)
std::vector<double> read_nodes(const std::string &path)
{
    Lines L(path);
    L.magic("ffea node file", "walrus node file");
    const long n = L.header(1, "num_nodes"), ns = L.header(2, "num_surface_nodes"),
               ni = L.header(3, "num_interior_nodes");
    if (ns + ni != n) raise(path + ": num_surface_nodes + num_interior_nodes != num_nodes");
    L.expect(4, "surface nodes:");
    std::vector<double> pos(3 * (size_t)n);
    size_t line = 5;
    for (long k = 0; k < n; k++) {
        if (k == ns) L.expect(line++, "interior nodes:");
        const std::vector<double> x = numbers(L, line++, 3);
        for (int c = 0; c < 3; c++) pos[3 * (size_t)k + c] = x[c];
    }
    return pos;
}

// Blob::load_topology: 10 node indices per element, bounds-checked
std::vector<int32_t> read_topology(const std::string &path, long num_nodes)
{
    Lines L(path);
    L.magic("ffea topology file", "walrus topology file");
    const long ne = L.header(1, "num_elements"), ns = L.header(2, "num_surface_elements");
    L.header(3, "num_interior_elements");
    L.expect(4, "surface elements:");
    std::vector<int32_t> topo(10 * (size_t)ne);
    size_t line = 5;
    for (long k = 0; k < ne; k++) {
        if (k == ns) L.expect(line++, "interior elements:");
        std::stringstream ss(L.at(line++));
        for (int j = 0; j < 10; j++) {
            long v = -1;
            if (!(ss >> v)) raise(path + ": element " + std::to_string(k) + " needs 10 node indices");
            if (v < 0 || v >= num_nodes) raise(path + ": element " + std::to_string(k) + " references node " +
                                               std::to_string(v) + ", out of bounds");
            topo[10 * (size_t)k + j] = (int32_t)v;
        }
    }
    return topo;
}

// Blob::load_material_params: density, shear and bulk viscosity, shear and
// bulk modulus, dielectric per element -> (rho, A, B, G, E) in meso units as
// src/Blob.cpp:2862-2867 computes them (the second viscosity coefficient
// subtracts the SI shear viscosity from the meso bulk viscosity, kept as is)
std::vector<double> read_material(const std::string &path, long num_elements)
{
    Lines L(path);
    L.magic("ffea material params file", "walrus material params file");
    const long ne = L.header(1, "num_elements");
    if (ne != num_elements) raise(path + ": element count does not match the topology");
    std::vector<double> mat(5 * (size_t)ne);
    for (long k = 0; k < ne; k++) {
        const std::vector<double> m = numbers(L, 2 + (size_t)k, 6);
        double *o = &mat[5 * (size_t)k];
        o[0] = m[0] * kMesoVolume / kMesoMass;
        o[1] = m[1] / (kMesoPressure * kMesoTime);
        o[2] = m[2] / (kMesoPressure * kMesoTime) - (2.0 / 3.0) * m[1];
        o[3] = m[3] / kMesoPressure;
        o[4] = m[4] / kMesoPressure;
    }
    return mat;
}

// Blob::load_stokes_params: one radius per node (file units)
std::vector<double> read_stokes(const std::string &path, long num_nodes)
{
    Lines L(path);
    L.magic("ffea stokes radii file", "walrus stokes radii file");
    const long n = L.header(1, "num_nodes");
    if (n != num_nodes) raise(path + ": node count does not match the node file");
    std::vector<double> r((size_t)n);
    for (long k = 0; k < n; k++) r[(size_t)k] = numbers(L, 2 + (size_t)k, 1)[0];
    return r;
}

// Blob::load_pinned_nodes
std::vector<int32_t> read_pin(const std::string &path, long num_nodes)
{
    Lines L(path);
    L.magic("ffea pinned nodes file", "walrus pinned nodes file");
    const long n = L.header(1, "num_pinned_nodes");
    L.expect(2, "pinned nodes:");
    std::vector<int32_t> p((size_t)n);
    for (long k = 0; k < n; k++) {
        std::stringstream ss(L.at(3 + (size_t)k));
        long v = -1;
        ss >> v;
        if (v < 0 || v >= num_nodes) raise(path + ": pinned node " + std::to_string(v) + " out of bounds");
        p[(size_t)k] = (int32_t)v;
    }
    return p;
}

struct Blob {
    std::vector<double> pos, vel, mat, drag;
    std::vector<int32_t> topo, pinned;
    int32_t solver = FFEA_GPU_SOLVER_NOMASS;
};

}  // namespace

struct ffea_gpu_script {
    ffea_gpu_script_params p;
    std::vector<Blob> blobs;
};

namespace {

// SimulationParams::assign for one <param> tag (src/SimulationParams.cpp:209-541)
void assign(ffea_gpu_script_params &p, const std::string &dir, const std::string &key, const std::string &v,
            std::vector<int> &confs, std::vector<int> &states)
{
    static const char *accepted[] = {
        "kappa", "dielec_ext", "epsilon_0", "es_update", "es_N_x", "es_N_y", "es_N_z", "es_h", "inc_self_ssint",
        "inc_self_vdw", "ssint_type", "vdw_type", "ssint_cutoff", "vdw_cutoff", "steric_factor",
        "vdw_steric_factor", "steric_dr", "vdw_steric_dr", "move_into_box", "wall_x_1", "wall_x_2", "wall_y_1",
        "wall_y_2", "wall_z_1", "wall_z_2", "ssint_in_fname", "vdw_in_fname", "ssint_forcefield_params",
        "vdw_forcefield_params", "lj_params", "ljparams", "kinetics_out_fname", "det_measurement_out_fname",
        "beads_out_fname", "bsite_in_fname", "kinetics_update", "force_pbc", "stress_out_fname", "calc_steric"};
    // switches of work outside the blob update: accepted only when off
    static const char *outside[] = {"calc_ssint", "calc_vdw", "calc_es", "calc_kinetics", "calc_preComp",
                                    "calc_springs", "calc_ctforces", "sticky_wall_xz"};
    if (key == "restart") p.restart = to_int(v, key);
    else if (key == "dt") p.dt = to_double(v, key) / kMesoTime;
    else if (key == "epsilon") {
        const double e = to_double(v, key);
        p.epsilon2 = e * e;
    } else if (key == "num_steps") p.num_steps = (int64_t)to_double(v, key);
    else if (key == "max_iterations_cg") p.max_iterations_cg = to_int(v, key);
    else if (key == "check") p.check = (int32_t)to_double(v, key);
    else if (key == "num_blobs") p.num_blobs = to_int(v, key);
    else if (key == "num_rods" || key == "num_couplings") {
        if (to_int(v, key) != 0) raise(key + " = " + v + ": rods are outside the GPU blob update");
    } else if (key == "num_conformations" || key == "num_states") {
        std::vector<int> &dst = key == "num_conformations" ? confs : states;
        dst.clear();
        for (double x : to_list(v, key)) dst.push_back((int)x);
    } else if (key == "rng_seed") {
        if (v == "time") raise("rng_seed = time: give a fixed seed (a GPU run is reproducible from it)");
        p.rng_seed = to_int(v, key);
    } else if (key == "kT") p.kT = to_double(v, key) / kMesoEnergy;
    else if (key == "calc_noise") p.calc_noise = to_int(v, key);
    else if (key == "calc_stokes" || key == "do_stokes") p.calc_stokes = to_int(v, key);
    else if (key == "stokes_visc") p.stokes_visc = to_double(v, key) / (kMesoPressure * kMesoTime);
    else if (key == "trajectory_out_fname") copy_name(p.trajectory_out_fname, join(dir, v));
    else if (key == "measurement_out_fname") copy_name(p.measurement_out_fname, join(dir, v));
    else if (key == "checkpoint_in") copy_name(p.checkpoint_in, join(dir, v));
    else if (key == "checkpoint_out") copy_name(p.checkpoint_out, join(dir, v));
    else {
        for (const char *k : outside)
            if (key == k) {
                if (to_int(v, key) != 0)
                    raise(key + " = " + v + " switches on work outside the GPU blob update (set it to 0)");
                return;
            }
        for (const char *k : accepted)
            if (key == k) return;
        raise("'" + key + "' is not a recognised parameter");
    }
}

std::unique_ptr<ffea_gpu_script> load(const char *path)
{
    const std::string spath(path);
    const size_t slash = spath.rfind('/');
    const std::string dir = slash == std::string::npos ? "" : spath.substr(0, slash);
    std::string base = slash == std::string::npos ? spath : spath.substr(slash + 1);
    const std::string stem = base.rfind('.') == std::string::npos ? base : base.substr(0, base.rfind('.'));
    const std::vector<std::string> script = script_lines(spath);

    std::unique_ptr<ffea_gpu_script> s(new ffea_gpu_script());
    ffea_gpu_script_params &p = s->p;
    std::memset(&p, 0, sizeof(p));
    // SimulationParams::SimulationParams (src/SimulationParams.cpp:26-77)
    p.dt = 1e-14 / kMesoTime;
    p.num_steps = (int64_t)1e11;
    p.check = 10000;
    p.kT = 4.11e-21 / kMesoEnergy;
    p.max_iterations_cg = 1000;
    p.epsilon2 = 0.01;
    p.rng_seed = -1;
    p.calc_noise = 1;
    p.calc_stokes = 1;
    p.stokes_visc = 1e-3 / (kMesoPressure * kMesoTime);
    p.restart = -1;
    std::vector<int> confs, states;

    std::vector<std::string> block;
    if (!extract_block(script, "param", 0, block)) raise("no <param> block");
    for (const std::string &l : block) {
        std::string k, v;
        parse_tag(l, k, v);
        assign(p, dir, k, v, confs, states);
    }
    // SimulationParams::validate (src/SimulationParams.cpp:580-720), the checks the path needs
    if (p.restart != 0 && p.restart != 1) raise("'restart' must be 0 or 1");
    if (p.restart == 1 && !p.checkpoint_in[0]) raise("restart = 1 needs a checkpoint_in file");
    if (p.num_steps < 0) raise("'num_steps' must be >= 0");
    if (p.num_blobs <= 0) raise("'num_blobs' must be > 0");
    if (p.rng_seed < 0) raise("'rng_seed' is required");
    if (p.check <= 0) raise("'check' must be > 0");
    for (int c : confs)
        if (c != 1) raise("num_conformations other than 1 are outside the GPU blob update");
    for (int c : states)
        if (c != 1) raise("num_states other than 1 are outside the GPU blob update");
    // output names FFEA derives from the script name when none is given
    if (!p.trajectory_out_fname[0]) copy_name(p.trajectory_out_fname, join(dir, stem + ".ftj"));
    if (!p.measurement_out_fname[0]) copy_name(p.measurement_out_fname, join(dir, stem + ".fm"));
    if (!p.checkpoint_out[0]) copy_name(p.checkpoint_out, join(dir, stem + ".fcp"));
    if (std::strcmp(p.checkpoint_out, p.checkpoint_in) == 0)
        raise("checkpoint_in and checkpoint_out must differ");

    std::vector<std::string> system;
    if (!extract_block(script, "system", 0, system)) raise("no <system> block");
    for (int i = 0; i < p.num_blobs; i++) {
        std::vector<std::string> bv, conf;
        if (!extract_block(system, "blob", i, bv)) raise("blob " + std::to_string(i) + ": no <blob> block");
        const bool as_conf = !extract_block(bv, "conformation", 0, conf);
        if (as_conf) conf = bv;
        std::vector<std::string> conf2;
        if (!as_conf && extract_block(bv, "conformation", 1, conf2))
            raise("blob " + std::to_string(i) + ": several conformations are outside the GPU blob update");
        std::string nodes, topo, mat, stokes, pin;
        for (const std::string &l : conf) {
            std::string k, v;
            parse_tag(l, k, v);
            if (k == "motion_state") {
                if (v != "DYNAMIC") raise("blob " + std::to_string(i) + ": motion_state " + v +
                                          " is outside the GPU blob update (DYNAMIC only)");
            } else if (k == "nodes") nodes = join(dir, v);
            else if (k == "topology") topo = join(dir, v);
            else if (k == "material") mat = join(dir, v);
            else if (k == "stokes") stokes = join(dir, v);
            else if (k == "pin") pin = join(dir, v);
            else if (k == "surface" || k == "ssint" || k == "vdw" || k == "binding_sites" || k == "beads") {
                // files of the interactions and kinetics, not read by the blob update
            } else if (as_conf && (k == "centroid" || k == "centroid_pos" || k == "rotation" || k == "solver" ||
                                   k == "scale" || k == "translate" || k == "velocity" || k == "calc_compress" ||
                                   k == "compress" || k == "conformation" || k == "/conformation")) {
                // blob-level tags, read below
            } else {
                raise("blob " + std::to_string(i) + ": unrecognised conformation tag '" + k + "'");
            }
        }
        if (nodes.empty() || topo.empty() || mat.empty())
            raise("blob " + std::to_string(i) + ": nodes, topology and material files are required");
        double scale = 0.0;
        bool has_scale = false, has_centroid = false, has_velocity = false;
        std::vector<double> centroid, velocity;
        Blob b;
        for (const std::string &l : bv) {
            std::string k, v;
            parse_tag(l, k, v);
            if (k == "solver") {
                if (v == "CG") b.solver = FFEA_GPU_SOLVER_MASS;
                else if (v == "CG_nomass") b.solver = FFEA_GPU_SOLVER_NOMASS;
                else if (v == "masslumped") b.solver = FFEA_GPU_SOLVER_LUMPED;
                else if (v == "direct") raise("blob " + std::to_string(i) + ": the direct solver is not supported");
                else raise("blob " + std::to_string(i) + ": unrecognised solver '" + v + "'");
            } else if (k == "scale") {
                scale = to_double(v, k) / kMesoLength;  // src/World.cpp:2564-2567
                has_scale = true;
            } else if (k == "centroid" || k == "centroid_pos") {
                centroid = to_list(v, k);
                if (centroid.size() != 3) raise("blob " + std::to_string(i) + ": centroid needs 3 values");
                has_centroid = true;
            } else if (k == "velocity") {
                velocity = to_list(v, k);
                if (velocity.size() != 3) raise("blob " + std::to_string(i) + ": velocity needs 3 values");
                for (double &x : velocity) x /= kMesoVelocity;
                has_velocity = true;
            } else if (k == "rotation" || k == "translate") {
                raise("blob " + std::to_string(i) + ": '" + k + "' is not supported by this front end");
            } else if (k == "calc_compress") {
                if (to_double(v, k) != 0.0) raise("blob " + std::to_string(i) + ": calc_compress is not supported");
            }
        }
        if (!has_scale) raise("blob " + std::to_string(i) + ": scale not set");
        // Blob::config loads and scales (src/Blob.cpp:2495-2497, 2925), Blob::init
        // sets the Stokes drag 6 pi eta r (src/Blob.cpp:408-412)
        b.pos = read_nodes(nodes);
        const long nn = (long)(b.pos.size() / 3);
        for (double &x : b.pos) x *= scale;
        b.topo = read_topology(topo, nn);
        const long ne = (long)(b.topo.size() / 10);
        b.mat = read_material(mat, ne);
        b.drag.assign((size_t)nn, 0.0);
        if (!stokes.empty()) {
            const std::vector<double> r = read_stokes(stokes, nn);
            if (p.calc_stokes == 1)
                for (long k = 0; k < nn; k++) b.drag[(size_t)k] = 6.0 * kPi * p.stokes_visc * (r[(size_t)k] * scale);
        } else if (p.calc_stokes == 1) {
            raise("blob " + std::to_string(i) + ": calc_stokes = 1 needs a stokes file");
        }
        if (!pin.empty()) b.pinned = read_pin(pin, nn);
        // World::read_and_build_system after Blob::init: the node centroid
        // moved to centroid * scale (Blob::position, src/Blob.cpp:886-922),
        // velocities set (Blob::velocity_all)
        if (has_centroid && nn > 0) {
            double c[3] = {0.0, 0.0, 0.0};
            for (long k = 0; k < nn; k++)
                for (int d = 0; d < 3; d++) c[d] += b.pos[3 * (size_t)k + d];
            for (int d = 0; d < 3; d++) {
                c[d] *= (1.0 / nn);
                const double shift = centroid[d] * scale - c[d];
                for (long k = 0; k < nn; k++) b.pos[3 * (size_t)k + d] += shift;
            }
        }
        b.vel.assign(3 * (size_t)nn, 0.0);
        if (has_velocity)
            for (long k = 0; k < nn; k++)
                for (int d = 0; d < 3; d++) b.vel[3 * (size_t)k + d] = velocity[d];
        s->blobs.push_back(std::move(b));
    }
    return s;
}

int fail(const std::string &m)
{
    ffea::set_last_error(m.c_str());
    return FFEA_GPU_ERROR;
}

}  // namespace

extern "C" {

int ffea_gpu_script_load(const char *path, ffea_gpu_script_t **out)
{
    if (!path || !out) return fail("null argument");
    *out = nullptr;
    try {
        *out = load(path).release();
    } catch (const Error &e) {
        return fail("script " + std::string(path) + ": " + e.msg);
    } catch (const std::exception &e) {
        return fail("script " + std::string(path) + ": " + e.what());
    }
    return FFEA_GPU_OK;
}

void ffea_gpu_script_free(ffea_gpu_script_t *s) { delete s; }

int ffea_gpu_script_get_params(const ffea_gpu_script_t *s, ffea_gpu_script_params *out)
{
    if (!s || !out) return fail("null argument");
    *out = s->p;
    return FFEA_GPU_OK;
}

int ffea_gpu_script_get_blob(const ffea_gpu_script_t *s, int32_t blob, ffea_gpu_mesh *mesh, ffea_gpu_params *params)
{
    if (!s || !mesh || !params) return fail("null argument");
    if (blob < 0 || blob >= (int32_t)s->blobs.size()) return fail("blob index out of range");
    const Blob &b = s->blobs[(size_t)blob];
    mesh->num_nodes = (int32_t)(b.pos.size() / 3);
    mesh->num_elements = (int32_t)(b.topo.size() / 10);
    mesh->pos = b.pos.data();
    mesh->vel = b.vel.data();
    mesh->topology = b.topo.data();
    mesh->material = b.mat.data();
    mesh->stokes_drag = b.drag.data();
    mesh->num_pinned = (int32_t)b.pinned.size();
    mesh->pinned = b.pinned.empty() ? nullptr : b.pinned.data();
    const ffea_gpu_script_params &p = s->p;
    params->dt = p.dt;
    params->kT = p.kT;
    params->epsilon2 = p.epsilon2;
    params->max_iterations_cg = p.max_iterations_cg;
    params->calc_noise = p.calc_noise;
    params->calc_stokes = p.calc_stokes;
    params->solver = b.solver;
    params->precision = FFEA_GPU_PRECISION_MIXED;
    params->rng_seed = p.rng_seed;
    params->true_residual = 1;
    params->preconditioner = FFEA_GPU_PRECOND_JACOBI;
    return FFEA_GPU_OK;
}

int ffea_gpu_script_create(const ffea_gpu_script_t *s, int32_t precision, int32_t preconditioner,
                           int32_t true_residual, ffea_gpu_t **out)
{
    if (!s || !out) return fail("null argument");
    const int32_t n = (int32_t)s->blobs.size();
    std::vector<ffea_gpu_mesh> meshes((size_t)n);
    std::vector<ffea_gpu_params> params((size_t)n);
    for (int32_t i = 0; i < n; i++) {
        if (ffea_gpu_script_get_blob(s, i, &meshes[(size_t)i], &params[(size_t)i]) != FFEA_GPU_OK)
            return FFEA_GPU_ERROR;
        params[(size_t)i].precision = precision;
        params[(size_t)i].preconditioner = preconditioner;
        params[(size_t)i].true_residual = true_residual;
    }
    // one RNG stream per blob seeded from the script's rng_seed, as
    // World::init seeds a one-thread run's blobs in turn (FFEA_GPU_RNG_SHARED)
    return ffea_gpu_create_batch(n, meshes.data(), params.data(), FFEA_GPU_RNG_SHARED, out);
}

}  // extern "C"

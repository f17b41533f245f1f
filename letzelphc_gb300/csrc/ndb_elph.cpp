// ndb.elph writer: the reference's variables (src/elph/elph_driver.c:152-187,
// src/io/write_basic_data.c:15-215) in the netCDF classic 64-bit-offset
// format (CDF-2).  Layout of the format: a header (magic "CDF\x02", record
// count, dimension list, global attribute list, variable list with each
// variable's dimension ids, type, padded size and 8-byte file offset) and
// then every fixed-size variable contiguously in row-major order, big-endian,
// padded to 4 bytes.  elph_mat is the last variable, so it may exceed 4 GiB.
#include <fcntl.h>
#include <unistd.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/lelph_ndb.h"

namespace
{
enum NcType
{
    NC_CHAR = 2,
    NC_INT = 4,
    NC_FLOAT = 5,
    NC_DOUBLE = 6
};

struct Var
{
    std::string name;
    std::vector<int> dims;  // dimension ids
    int type;
    unsigned long long bytes = 0;  // unpadded size
    unsigned long long begin = 0;
};

int type_size(int t) { return t == NC_CHAR ? 1 : (t == NC_DOUBLE ? 8 : 4); }
unsigned long long pad4(unsigned long long n) { return (n + 3) & ~3ull; }

struct Header
{
    std::vector<std::pair<std::string, unsigned long long>> dims;
    std::vector<Var> vars;

    int dim(const std::string& name, unsigned long long len)
    {
        for (size_t i = 0; i < dims.size(); ++i)
            if (dims[i].first == name) return dims[i].second == len ? (int)i : -1;
        dims.emplace_back(name, len);
        return (int)dims.size() - 1;
    }
    // def_ncVar (src/io/nc4_def_var.c:10-71): dimensions by name, a name reused
    // with another length is an error
    bool var(const std::string& name, int type, const std::vector<std::pair<std::string, unsigned long long>>& d)
    {
        Var v;
        v.name = name;
        v.type = type;
        unsigned long long n = type_size(type);
        for (auto& x : d)
        {
            int id = dim(x.first, x.second);
            if (id < 0) return false;
            v.dims.push_back(id);
            n *= x.second;
        }
        v.bytes = n;
        vars.push_back(v);
        return true;
    }
};

void put_u32(std::vector<unsigned char>& b, uint32_t v)
{
    for (int s = 24; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
}
void put_u64(std::vector<unsigned char>& b, uint64_t v)
{
    for (int s = 56; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
}
void put_name(std::vector<unsigned char>& b, const std::string& s)
{
    put_u32(b, (uint32_t)s.size());
    b.insert(b.end(), s.begin(), s.end());
    while (b.size() % 4) b.push_back(0);
}

std::vector<unsigned char> encode(const Header& h)
{
    std::vector<unsigned char> b = {'C', 'D', 'F', 2};
    put_u32(b, 0);  // no record variables
    put_u32(b, 0x0A);
    put_u32(b, (uint32_t)h.dims.size());
    for (auto& d : h.dims)
    {
        put_name(b, d.first);
        put_u32(b, (uint32_t)d.second);
    }
    put_u32(b, 0);  // no global attributes
    put_u32(b, 0);
    put_u32(b, 0x0B);
    put_u32(b, (uint32_t)h.vars.size());
    for (auto& v : h.vars)
    {
        put_name(b, v.name);
        put_u32(b, (uint32_t)v.dims.size());
        for (int id : v.dims) put_u32(b, (uint32_t)id);
        put_u32(b, 0);  // no attributes
        put_u32(b, 0);
        put_u32(b, (uint32_t)v.type);
        const unsigned long long vs = pad4(v.bytes);
        put_u32(b, vs > 0xFFFFFFFCull ? 0xFFFFFFFFu : (uint32_t)vs);
        put_u64(b, v.begin);
    }
    return b;
}

// big-endian element encoders
void be_double(unsigned char* p, double x)
{
    uint64_t u;
    memcpy(&u, &x, 8);
    for (int i = 0; i < 8; ++i) p[i] = (unsigned char)(u >> (56 - 8 * i));
}
void be_float(unsigned char* p, float x)
{
    uint32_t u;
    memcpy(&u, &x, 4);
    for (int i = 0; i < 4; ++i) p[i] = (unsigned char)(u >> (24 - 8 * i));
}
void be_int(unsigned char* p, int32_t x)
{
    const uint32_t u = (uint32_t)x;
    for (int i = 0; i < 4; ++i) p[i] = (unsigned char)(u >> (24 - 8 * i));
}
}  // namespace

struct lelph_ndb
{
    int fd = -1;
    Header h;
    lelph_ndb_desc d;
    int io_type = NC_DOUBLE;
    int v_eig = -1, v_freq = -1, v_elph = -1;

    const Var& var(int i) const { return h.vars[(size_t)i]; }
    int find(const char* name) const
    {
        for (size_t i = 0; i < h.vars.size(); ++i)
            if (h.vars[i].name == name) return (int)i;
        return -1;
    }
    bool write_at(unsigned long long off, const void* p, size_t n)
    {
        const unsigned char* c = (const unsigned char*)p;
        while (n)
        {
            ssize_t w = pwrite(fd, c, n, (off_t)off);
            if (w <= 0) return false;
            c += w;
            n -= (size_t)w;
            off += (unsigned long long)w;
        }
        return true;
    }
    // real values of a whole variable (or a slice starting `first` elements in)
    bool put_real(int iv, unsigned long long first, const double* x, size_t n)
    {
        const int es = type_size(io_type);
        std::vector<unsigned char> buf(n * es);
        for (size_t i = 0; i < n; ++i)
        {
            if (io_type == NC_DOUBLE)
                be_double(&buf[i * 8], x ? x[i] : 0.0);
            else
                be_float(&buf[i * 4], x ? (float)x[i] : 0.0f);
        }
        return write_at(var(iv).begin + first * es, buf.data(), buf.size());
    }
    bool put_int(int iv, const int* x, size_t n)
    {
        std::vector<unsigned char> buf(n * 4);
        for (size_t i = 0; i < n; ++i) be_int(&buf[i * 4], x[i]);
        return write_at(var(iv).begin, buf.data(), buf.size());
    }
};

extern "C" int lelph_ndb_create(const char* path, const lelph_ndb_desc* dp, lelph_ndb** out)
{
    if (!path || !dp || !out) return -1;
    *out = nullptr;
    const lelph_ndb_desc& d = *dp;
    if (d.nq_BZ <= 0 || d.nq_iBZ <= 0 || d.nkpts_BZ <= 0 || d.nmodes <= 0 || d.natom <= 0 || d.nspin <= 0 ||
        d.nbnds <= 0 || d.nph_sym <= 0 || d.nmodes != 3 * d.natom || !d.kpoints || !d.qpoints || !d.qpoints_iBZ ||
        !d.qmap || !d.kmap || !d.sym_Rmat || !d.sym_tau || !d.sym_time_rev || !d.kernel)
        return -1;
    lelph_ndb* f = new (std::nothrow) lelph_ndb();
    if (!f) return -2;
    f->d = d;
    f->io_type = d.io_double ? NC_DOUBLE : NC_FLOAT;
    const int R = f->io_type;
    typedef unsigned long long u;
    const u nq = (u)d.nq_BZ, nm = (u)d.nmodes, nk = (u)d.nkpts_BZ, nb = (u)d.nbnds;
    Header& h = f->h;
    const std::string conv = d.kminusq ? "yambo" : "standard";
    bool ok = true;
    // elph_driver.c:152-187
    ok = ok && h.var("POLARIZATION_VECTORS", R, {{"nq", nq}, {"nmodes", nm}, {"atom", nm / 3}, {"pol", 3}, {"re_im", 2}});
    ok = ok && h.var("FREQ", R, {{"nq", nq}, {"nmodes", nm}});
    // write_basic_data.c:29-177
    ok = ok && h.var("kpoints", R, {{"nk", nk}, {"pol", 3}});
    ok = ok && h.var("qpoints", R, {{"nq", nq}, {"pol", 3}});
    ok = ok && h.var("qpoints_iBZ", R, {{"nq_iBZ", (u)d.nq_iBZ}, {"pol", 3}});
    ok = ok && h.var("qmap", NC_INT, {{"nq", nq}, {"dim_two", 2}});
    ok = ok && h.var("kmap", NC_INT, {{"nk", nk}, {"dim_two", 2}});
    ok = ok && h.var("bands", NC_INT, {{"two_scalars", 2}});
    ok = ok && h.var("number_of_phonon_symmetries", NC_INT, {{"scalar", 1}});
    ok = ok && h.var("time_reversal_phonon", NC_INT, {{"scalar", 1}});
    ok = ok && h.var("symmetry_matrices", R, {{"nsym_ph", (u)d.nph_sym}, {"pol", 3}, {"pol", 3}});
    ok = ok && h.var("fractional_translation", R, {{"nsym_ph", (u)d.nph_sym}, {"pol", 3}});
    ok = ok && h.var("kernel", NC_CHAR, {{"kernel_str_size", (u)strlen(d.kernel) + 1}});
    ok = ok && h.var("convention", NC_CHAR, {{"convention_str_size", (u)conv.size() + 1}});
    ok = ok && h.var("epsilon", R, {{"pol", 3}, {"pol", 3}});
    ok = ok && h.var("Born_charges", R, {{"natoms", (u)d.natom}, {"pol", 3}, {"pol", 3}});
    ok = ok && h.var("Quadrupole_tensor", R, {{"natoms", (u)d.natom}, {"pol", 3}, {"pol", 3}, {"pol", 3}});
    // last: the only variable allowed past 4 GiB in this format
    ok = ok && h.var("elph_mat", R,
                     {{"nq", nq}, {"nk", nk}, {"nmodes", nm}, {"nspin", (u)d.nspin}, {"initial_band", nb},
                      {"final_band_PH_abs", nb}, {"re_im", 2}});
    if (!ok)
    {
        delete f;
        return -1;
    }
    for (size_t i = 0; i + 1 < h.vars.size(); ++i)
        if (pad4(h.vars[i].bytes) > 0xFFFFFFFCull)
        {
            delete f;
            return -1;  // only the last variable may exceed 4 GiB in CDF-2
        }
    // offsets: the header length does not depend on them
    unsigned long long off = encode(h).size();
    for (auto& v : h.vars)
    {
        v.begin = off;
        off += pad4(v.bytes);
    }
    f->v_eig = f->find("POLARIZATION_VECTORS");
    f->v_freq = f->find("FREQ");
    f->v_elph = f->find("elph_mat");
    f->fd = open(path, O_CREAT | O_TRUNC | O_RDWR, 0644);
    if (f->fd < 0)
    {
        delete f;
        return -8;
    }
    const std::vector<unsigned char> hdr = encode(h);
    ok = f->write_at(0, hdr.data(), hdr.size()) && ftruncate(f->fd, (off_t)off) == 0;
    // basic data
    std::vector<double> R9((size_t)9 * d.nph_sym), T3((size_t)3 * d.nph_sym);
    int trev = 0;
    for (int s = 0; s < d.nph_sym; ++s)
    {
        memcpy(&R9[9 * (size_t)s], d.sym_Rmat + 9 * (size_t)s, 9 * sizeof(double));
        memcpy(&T3[3 * (size_t)s], d.sym_tau + 3 * (size_t)s, 3 * sizeof(double));
        if (d.sym_time_rev[s]) trev = 1;
    }
    const int bands[2] = {d.start_band, d.end_band}, nsym = d.nph_sym;
    ok = ok && f->put_real(f->find("kpoints"), 0, d.kpoints, 3 * nk);
    ok = ok && f->put_real(f->find("qpoints"), 0, d.qpoints, 3 * nq);
    ok = ok && f->put_real(f->find("qpoints_iBZ"), 0, d.qpoints_iBZ, 3 * (size_t)d.nq_iBZ);
    ok = ok && f->put_int(f->find("qmap"), d.qmap, 2 * nq);
    ok = ok && f->put_int(f->find("kmap"), d.kmap, 2 * nk);
    ok = ok && f->put_int(f->find("bands"), bands, 2);
    ok = ok && f->put_int(f->find("number_of_phonon_symmetries"), &nsym, 1);
    ok = ok && f->put_int(f->find("time_reversal_phonon"), &trev, 1);
    ok = ok && f->put_real(f->find("symmetry_matrices"), 0, R9.data(), R9.size());
    ok = ok && f->put_real(f->find("fractional_translation"), 0, T3.data(), T3.size());
    ok = ok && f->write_at(f->var(f->find("kernel")).begin, d.kernel, strlen(d.kernel) + 1);
    ok = ok && f->write_at(f->var(f->find("convention")).begin, conv.c_str(), conv.size() + 1);
    ok = ok && f->put_real(f->find("epsilon"), 0, d.epsilon, 9);
    ok = ok && f->put_real(f->find("Born_charges"), 0, d.Zborn, 9 * (size_t)d.natom);
    ok = ok && f->put_real(f->find("Quadrupole_tensor"), 0, d.Qpole, 27 * (size_t)d.natom);
    if (!ok)
    {
        close(f->fd);
        delete f;
        return -8;
    }
    // the caller's arrays are not kept
    f->d.kpoints = f->d.qpoints = f->d.qpoints_iBZ = f->d.sym_Rmat = f->d.sym_tau = nullptr;
    f->d.qmap = f->d.kmap = f->d.sym_time_rev = nullptr;
    f->d.kernel = nullptr;
    f->d.epsilon = f->d.Zborn = f->d.Qpole = nullptr;
    *out = f;
    return 0;
}

extern "C" int lelph_ndb_put_elph(lelph_ndb* f, int iq, int k0, int nk, const void* g, int c64)
{
    if (!f || !g || iq < 0 || iq >= f->d.nq_BZ || k0 < 0 || nk < 0 || k0 + nk > f->d.nkpts_BZ) return -1;
    const size_t slice = (size_t)f->d.nmodes * f->d.nspin * f->d.nbnds * f->d.nbnds * 2;  // reals per k
    const int es = type_size(f->io_type);
    std::vector<unsigned char> buf(slice * es);
    for (int k = 0; k < nk; ++k)
    {
        for (size_t i = 0; i < slice; ++i)
        {
            const double x = c64 ? (double)((const float*)g)[(size_t)k * slice + i] : ((const double*)g)[(size_t)k * slice + i];
            if (f->io_type == NC_DOUBLE)
                be_double(&buf[i * 8], x);
            else
                be_float(&buf[i * 4], (float)x);
        }
        const unsigned long long first = ((unsigned long long)iq * f->d.nkpts_BZ + (unsigned long long)(k0 + k)) * slice;
        if (!f->write_at(f->var(f->v_elph).begin + first * es, buf.data(), buf.size())) return -8;
    }
    return 0;
}

extern "C" int lelph_ndb_put_phonon(lelph_ndb* f, int iq, const double* eig, const double* omega)
{
    if (!f || iq < 0 || iq >= f->d.nq_BZ) return -1;
    const size_t ne = (size_t)f->d.nmodes * f->d.nmodes * 2;
    if (eig && !f->put_real(f->v_eig, (unsigned long long)iq * ne, eig, ne)) return -8;
    if (omega && !f->put_real(f->v_freq, (unsigned long long)iq * f->d.nmodes, omega, (size_t)f->d.nmodes)) return -8;
    return 0;
}

extern "C" int lelph_ndb_close(lelph_ndb* f)
{
    if (!f) return -1;
    int rc = 0;
    if (f->fd >= 0)
    {
        if (fsync(f->fd) != 0) rc = -8;
        if (close(f->fd) != 0) rc = -8;
    }
    delete f;
    return rc;
}

/*
 * nbodygo.hpp - C++ host mirror of the reference's runner/body API over the
 * C ABI of libnbgpu.so (nbgpu.h).
 *
 * The names, argument meanings and results follow the Go packages the GPU
 * cycle replaces, so code (and tests) written against them read the same:
 *
 *   Body, NewBody, Body::ApplyMods         cmd/body/body.go:34-89, 274-313
 *   ParseCollisionBehavior, ParseBoolean,  cmd/globals/globals.go:41-102
 *     SafeParseFloat
 *   BodyCollection (NewSimBodyCollection,  cmd/body/body_collection.go:45-305
 *     Enqueue(NewAdd), ModBody, GetBody,
 *     Count, GetArray)
 *   ModBodyResult                          cmd/grpcsimcb/grpcsimcb.go:8-20
 *   ComputationRunner (NewComputationRunner, cmd/runner/computation-runner.go:24-326
 *     SetTimeScaling, SetCoefficientOfRestitution, RemoveBodies, SetWorkers,
 *     RunOneComputation, TimeScaling, CoefficientOfRestitution, WorkerCount)
 *   NextId, Body::SetSun                   cmd/body/body.go:101-104, 315-328
 *   FromCsv                                cmd/sim/fromcsv.go:46-131
 *   ToCsv (snapshot in FromCsv's format; no counterpart in the reference)
 *
 * The body array lives on the GPU; strings (Name, Class), colour and light
 * intensity stay here, keyed by id.  The setters of the runner take effect at
 * the start of the next cycle, as the reference's 1-slot channels do.  Errors
 * of the C ABI surface as nbodygo::Error exceptions.
 */
#ifndef NBODYGO_HPP
#define NBODYGO_HPP

#include <atomic>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "nbgpu.h"

namespace nbodygo {

enum CollisionBehavior { None = NBG_NONE, Subsume = NBG_SUBSUME, Elastic = NBG_ELASTIC, Fragment = NBG_FRAGMENT };

enum BodyColor {
    Random, Black, White, Darkgray, Gray, Lightgray, Red, Green, Blue, Yellow, Magenta, Cyan, Orange, Brown, Pink
};

/* grpcsimcb.ModBodyResult */
enum ModBodyResult { NoMatch = 0, ModAll = 1, ModSome = 2, ModNone = 3 };

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline std::string lower(std::string s)
{
    for (char &c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}

/* globals.ParseCollisionBehavior: unknown strings give Elastic. */
inline CollisionBehavior ParseCollisionBehavior(const std::string &s)
{
    const char *names[] = {"none", "subsume", "elastic", "fragment"};
    for (int i = 0; i < 4; i++)
        if (lower(s) == names[i]) return (CollisionBehavior)i;
    return Elastic;
}

/* globals.ParseBoolean */
inline bool ParseBoolean(const std::string &s)
{
    const std::string l = lower(s);
    return l == "t" || l == "true" || l == "1" || l == "y" || l == "yes";
}

/* globals.ParseBodyColor: unknown strings give Random. */
inline BodyColor ParseBodyColor(const std::string &s)
{
    const char *names[] = {"random", "black", "white", "darkgray", "gray", "lightgray", "red", "green",
                           "blue", "yellow", "magenta", "cyan", "orange", "brown", "pink"};
    for (int i = 0; i < 15; i++)
        if (lower(s) == names[i]) return (BodyColor)i;
    return Random;
}

/* globals.SafeParseFloat: the parsed value, or cur when s is not a number
 * (strconv.ParseFloat accepts the whole string or nothing). */
inline double SafeParseFloat(const std::string &s, double cur)
{
    if (s.empty() || std::isspace((unsigned char)s[0])) return cur; /* strtod would skip it, Go does not */
    const char *b = s.c_str();
    char *end = nullptr;
    errno = 0;
    const double v = std::strtod(b, &end);
    if (end == b || *end != '\0') return cur;
    if (errno == ERANGE && std::isinf(v)) return cur; /* Go returns an error for out-of-range */
    return v;
}

/* The Body struct (body.go:34-52).  The private Go fields (r, fragmenting,
 * fragInfo, fx/fy/fz, collided) live on the device and are read back by
 * BodyCollection::GetBody. */
struct Body {
    int64_t Id = 0;
    std::string Name, Class;
    double X = 0, Y = 0, Z = 0, Vx = 0, Vy = 0, Vz = 0, Radius = 0, Mass = 0;
    double FragFactor = 0, FragStep = 0;
    CollisionBehavior Behavior = Elastic;
    BodyColor Color = Random;
    bool IsSun = false, Exists = true, WithTelemetry = false, Pinned = false;

    double intensity = 0;
    /* body.go:101-104 */
    void SetSun(double i)
    {
        IsSun = true;
        intensity = i;
    }

    /* body.go:274-313: property=value strings; unknown properties and parse
     * errors are ignored; always returns true. */
    bool ApplyMods(const std::vector<std::string> &mods)
    {
        for (const std::string &mod : mods) {
            const size_t eq = mod.find('=');
            if (eq == std::string::npos || mod.find('=', eq + 1) != std::string::npos) continue;
            std::string key = mod.substr(0, eq), val = mod.substr(eq + 1);
            for (char &c : key) c = (char)std::toupper((unsigned char)c);
            if (key == "X") X = SafeParseFloat(val, X);
            else if (key == "Y") Y = SafeParseFloat(val, Y);
            else if (key == "Z") Z = SafeParseFloat(val, Z);
            else if (key == "VX") Vx = SafeParseFloat(val, Vx);
            else if (key == "VY") Vy = SafeParseFloat(val, Vy);
            else if (key == "VZ") Vz = SafeParseFloat(val, Vz);
            else if (key == "MASS") Mass = SafeParseFloat(val, Mass);
            else if (key == "RADIUS") Radius = SafeParseFloat(val, Radius);
            else if (key == "FRAG-FACTOR") FragFactor = SafeParseFloat(val, FragFactor);
            else if (key == "FRAG-STEP") FragStep = SafeParseFloat(val, FragStep);
            else if (key == "COLLISION") Behavior = ParseCollisionBehavior(val);
            else if (key == "COLOR") {
                if (!IsSun) Color = ParseBodyColor(val); /* suns stay white */
            } else if (key == "TELEMETRY") WithTelemetry = ParseBoolean(val);
            else if (key == "EXISTS") Exists = ParseBoolean(val);
        }
        return true;
    }
};

/* body.NextId (body.go:315-328): one counter for the process, shared with the
 * ids the GPU gives fragments (ComputationRunner keeps the two in step). */
inline std::atomic<int64_t> &next_id_counter()
{
    static std::atomic<int64_t> c{0};
    return c;
}
inline int64_t NextId() { return next_id_counter().fetch_add(1); }
/* raises the counter to at least v */
inline void AdvanceNextId(int64_t v)
{
    int64_t cur = next_id_counter().load();
    while (cur < v && !next_id_counter().compare_exchange_weak(cur, v)) {
    }
}

/* body.NewBody (body.go:56-89) */
inline Body NewBody(int64_t id, double x, double y, double z, double vx, double vy, double vz, double mass,
                    double radius, CollisionBehavior behavior, BodyColor color, double fragFactor,
                    double fragStep, bool withTelemetry, const std::string &name, const std::string &cls,
                    bool pinned)
{
    Body b;
    b.Id = id;
    b.Name = name;
    b.Class = cls;
    b.X = x; b.Y = y; b.Z = z;
    b.Vx = vx; b.Vy = vy; b.Vz = vz;
    b.Mass = mass;
    b.Radius = radius;
    b.Behavior = behavior;
    b.Color = color;
    b.FragFactor = fragFactor;
    b.FragStep = fragStep;
    b.WithTelemetry = withTelemetry;
    b.Pinned = pinned;
    return b;
}

/* strconv.ParseBool: true for 1 t T TRUE true True, false for 0 f F FALSE
 * false False; anything else is an error (returns false in *ok) */
inline bool GoParseBool(const std::string &s, bool *ok)
{
    static const char *t[] = {"1", "t", "T", "TRUE", "true", "True"};
    static const char *f[] = {"0", "f", "F", "FALSE", "false", "False"};
    *ok = true;
    for (const char *v : t)
        if (s == v) return true;
    for (const char *v : f)
        if (s == v) return false;
    *ok = false;
    return false;
}

/* strconv.ParseFloat(s, 64) on the whole string; *ok = false on any error */
inline double GoParseFloat(const std::string &s, bool *ok)
{
    const double nan_marker = 0;
    *ok = false;
    if (s.empty() || std::isspace((unsigned char)s[0])) return nan_marker;
    const char *b = s.c_str();
    char *end = nullptr;
    errno = 0;
    const double v = std::strtod(b, &end);
    if (end == b || *end != '\0' || (errno == ERANGE && std::isinf(v))) return nan_marker;
    *ok = true;
    return v;
}

inline std::string TrimSpace(const std::string &s)
{
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) a++;
    while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
    return s.substr(a, b - a);
}

/* One record of encoding/csv with Comment '#' and FieldsPerRecord -1: comma
 * separated, RFC 4180 quotes ("" inside a quoted field; a quoted field may
 * span lines), lines starting with '#' and empty lines skipped.  Returns
 * false at end of input; a bare quote in an unquoted field is an error, as
 * in Go (the reference then stops the process; here Error is thrown). */
inline bool ReadCsvRecord(std::istream &in, std::vector<std::string> &fields)
{
    std::string line;
    for (;;) {
        if (!std::getline(in, line)) return false;
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (line.empty() || line[0] == '#') continue;
        break;
    }
    fields.clear();
    std::string cur;
    size_t i = 0;
    for (;;) {
        if (i < line.size() && line[i] == '"') {
            /* quoted field */
            i++;
            for (;;) {
                if (i >= line.size()) {
                    std::string next;
                    if (!std::getline(in, next)) throw Error(NBG_E_ARG, "csv: extraneous or missing \" in quoted-field");
                    if (!next.empty() && next.back() == '\r') next.pop_back();
                    cur += '\n';
                    line = next;
                    i = 0;
                    continue;
                }
                if (line[i] == '"') {
                    if (i + 1 < line.size() && line[i + 1] == '"') {
                        cur += '"';
                        i += 2;
                        continue;
                    }
                    i++;
                    break;
                }
                cur += line[i++];
            }
            if (i < line.size() && line[i] != ',') throw Error(NBG_E_ARG, "csv: extraneous \" in field");
        } else {
            while (i < line.size() && line[i] != ',') {
                if (line[i] == '"') throw Error(NBG_E_ARG, "csv: bare \" in non-quoted-field");
                cur += line[i++];
            }
        }
        fields.push_back(cur);
        cur.clear();
        if (i >= line.size()) break;
        i++; /* the comma */
        if (i >= line.size()) {
            fields.push_back("");
            break;
        }
    }
    return true;
}

/* sim.FromCsv (cmd/sim/fromcsv.go:46-131): fields x, y, z, vx, vy, vz, mass,
 * radius (required), is_sun, collision_behavior, color, fragmentation_factor,
 * fragmentation_step (optional, in that order).  A record whose required
 * fields are missing or whose present fields do not parse is skipped, as the
 * reference's recovered panic does: an empty optional field that is parsed
 * (is_sun, the two fragmentation values) does not parse, so such a record is
 * skipped too.  At most bodyCount records are kept; each body gets NextId().
 * An unreadable file gives an empty list. */
inline std::vector<Body> FromCsv(const std::string &csvPath, int bodyCount, CollisionBehavior defaultCollisionBehavior,
                                 BodyColor defaultBodyColor)
{
    std::vector<Body> bodies;
    std::ifstream in(csvPath);
    if (!in) return bodies;
    std::vector<std::string> f;
    for (int lines = 0; lines < bodyCount;) {
        if (!ReadCsvRecord(in, f)) break;
        if (f.size() < 8) continue;
        bool ok = true, o;
        double v[8];
        for (int k = 0; k < 8 && ok; k++) {
            v[k] = GoParseFloat(TrimSpace(f[k]), &o);
            ok = o;
        }
        if (!ok) continue;
        bool isSun = false;
        if (f.size() >= 9) {
            isSun = GoParseBool(TrimSpace(f[8]), &o);
            if (!o) continue;
        }
        CollisionBehavior cb = defaultCollisionBehavior;
        if (f.size() >= 10) cb = ParseCollisionBehavior(TrimSpace(f[9]));
        BodyColor color = defaultBodyColor;
        if (f.size() >= 11) color = ParseBodyColor(TrimSpace(f[10]));
        double fragFactor = 0, fragStep = 0;
        if (f.size() >= 12) {
            fragFactor = GoParseFloat(TrimSpace(f[11]), &o);
            if (!o) continue;
        }
        if (f.size() >= 13) {
            fragStep = GoParseFloat(TrimSpace(f[12]), &o);
            if (!o) continue;
        }
        Body b = NewBody(NextId(), v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], cb, color, fragFactor, fragStep,
                         false, "", "", false);
        if (isSun) b.SetSun(100);
        bodies.push_back(b);
        lines++;
    }
    return bodies;
}

/* Snapshot of bodies in FromCsv's 13-field format, every number written with
 * 17 significant digits, so FromCsv reads back the same values bit for bit
 * (ids come from NextId again).  Returns false if the file cannot be written. */
inline bool ToCsv(const std::string &path, const std::vector<Body> &bodies)
{
    static const char *beh[] = {"none", "subsume", "elastic", "fragment"};
    static const char *col[] = {"random", "black", "white", "darkgray", "gray", "lightgray", "red", "green",
                                "blue", "yellow", "magenta", "cyan", "orange", "brown", "pink"};
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    std::fprintf(f, "# x,y,z,vx,vy,vz,mass,radius,is_sun,collision_behavior,color,fragmentation_factor,"
                    "fragmentation_step\n");
    for (const Body &b : bodies)
        std::fprintf(f, "%.17g,%.17g,%.17g,%.17g,%.17g,%.17g,%.17g,%.17g,%s,%s,%s,%.17g,%.17g\n", b.X, b.Y, b.Z, b.Vx,
                     b.Vy, b.Vz, b.Mass, b.Radius, b.IsSun ? "true" : "false", beh[b.Behavior & 3],
                     col[(unsigned)b.Color < 15 ? b.Color : 0], b.FragFactor, b.FragStep);
    return std::fclose(f) == 0;
}

/* The numeric part of ApplyMods as an nbg_edit (the C ABI's ModBody). */
inline nbg_edit EditFromMods(int64_t id, const std::vector<std::string> &mods, const Body &before)
{
    Body after = before;
    after.ApplyMods(mods);
    nbg_edit e{};
    e.id = id;
    e.x = after.X; e.y = after.Y; e.z = after.Z;
    e.vx = after.Vx; e.vy = after.Vy; e.vz = after.Vz;
    e.mass = after.Mass; e.radius = after.Radius;
    e.frag_factor = after.FragFactor; e.frag_step = after.FragStep;
    e.collision = after.Behavior;
    e.telemetry = after.WithTelemetry;
    e.exists = after.Exists;
    e.mask = NBG_M_X | NBG_M_Y | NBG_M_Z | NBG_M_VX | NBG_M_VY | NBG_M_VZ | NBG_M_MASS | NBG_M_RADIUS |
             NBG_M_FRAG_FACTOR | NBG_M_FRAG_STEP | NBG_M_COLLISION | NBG_M_TELEMETRY | NBG_M_EXISTS;
    return e;
}

struct SoaBuffers {
    std::vector<int64_t> id, frag_fragments;
    std::vector<double> x, y, z, vx, vy, vz, radius, mass, ff, fs, r, fx, fy, fz, frr, frn, frm, fcx, fcy, fcz;
    std::vector<int32_t> collision;
    std::vector<uint32_t> flags;
    void resize(size_t n)
    {
        for (auto *v : {&id, &frag_fragments}) v->resize(n);
        for (auto *v : {&x, &y, &z, &vx, &vy, &vz, &radius, &mass, &ff, &fs, &r, &fx, &fy, &fz, &frr, &frn, &frm,
                        &fcx, &fcy, &fcz})
            v->resize(n);
        collision.resize(n);
        flags.resize(n);
    }
    nbg_soa soa()
    {
        nbg_soa s{};
        s.id = id.data(); s.x = x.data(); s.y = y.data(); s.z = z.data();
        s.vx = vx.data(); s.vy = vy.data(); s.vz = vz.data();
        s.radius = radius.data(); s.mass = mass.data();
        s.frag_factor = ff.data(); s.frag_step = fs.data();
        s.collision = collision.data(); s.flags = flags.data();
        s.r = r.data(); s.fx = fx.data(); s.fy = fy.data(); s.fz = fz.data();
        s.frag_radius = frr.data(); s.frag_new_radius = frn.data(); s.frag_mass = frm.data();
        s.frag_fragments = frag_fragments.data();
        s.frag_cx = fcx.data(); s.frag_cy = fcy.data(); s.frag_cz = fcz.data();
        return s;
    }
    void put(size_t k, const Body &b)
    {
        id[k] = b.Id; x[k] = b.X; y[k] = b.Y; z[k] = b.Z; vx[k] = b.Vx; vy[k] = b.Vy; vz[k] = b.Vz;
        radius[k] = b.Radius; mass[k] = b.Mass; ff[k] = b.FragFactor; fs[k] = b.FragStep;
        collision[k] = b.Behavior;
        flags[k] = (b.Exists ? NBG_F_EXISTS : 0u) | (b.IsSun ? NBG_F_IS_SUN : 0u) | (b.Pinned ? NBG_F_PINNED : 0u) |
                   (b.WithTelemetry ? NBG_F_TELEMETRY : 0u);
        r[k] = 1.0; fx[k] = fy[k] = fz[k] = 0;
        frr[k] = frn[k] = frm[k] = fcx[k] = fcy[k] = fcz[k] = 0;
        frag_fragments[k] = 0;
    }
    Body get(size_t k) const
    {
        Body b;
        b.Id = id[k]; b.X = x[k]; b.Y = y[k]; b.Z = z[k]; b.Vx = vx[k]; b.Vy = vy[k]; b.Vz = vz[k];
        b.Radius = radius[k]; b.Mass = mass[k]; b.FragFactor = ff[k]; b.FragStep = fs[k];
        b.Behavior = (CollisionBehavior)collision[k];
        b.Exists = flags[k] & NBG_F_EXISTS; b.IsSun = flags[k] & NBG_F_IS_SUN;
        b.Pinned = flags[k] & NBG_F_PINNED; b.WithTelemetry = flags[k] & NBG_F_TELEMETRY;
        return b;
    }
};

/* BodyCollection: the body array is the device copy of one nbg_ctx. */
class BodyCollection {
  public:
    /* NewSimBodyCollection (body_collection.go:45-68) */
    explicit BodyCollection(const std::vector<Body> &bodies, int precision = NBG_PRECISION_FP64, int device = 0)
    {
        nbg_ctx *c = nullptr;
        int rc = nbg_create(device, precision, (int64_t)bodies.size() + 1024, &c);
        if (rc != NBG_OK) throw Error(rc, nbg_last_error(nullptr));
        ctx_.reset(c);
        SoaBuffers b;
        b.resize(bodies.size());
        int64_t max_id = -1;
        for (size_t k = 0; k < bodies.size(); k++) {
            b.put(k, bodies[k]);
            remember(bodies[k]);
            if (bodies[k].Id > max_id) max_id = bodies[k].Id;
        }
        nbg_soa s = b.soa();
        check(nbg_set_bodies(ctx_.get(), &s, (int64_t)bodies.size()));
        AdvanceNextId(max_id + 1);
        check(nbg_set_next_id(ctx_.get(), next_id_counter().load()));
    }

    nbg_ctx *ctx() const { return ctx_.get(); }

    /* Enqueue(NewAdd(b)) (body_collection.go:82-88): appended by the next
     * Cycle, newest first.  Returns the id (NextId() when b.Id < 0). */
    int64_t EnqueueAdd(Body b)
    {
        if (b.Id < 0) b.Id = NextId();
        SoaBuffers s;
        s.resize(1);
        s.put(0, b);
        s.id[0] = b.Id;
        nbg_soa soa = s.soa();
        int64_t id = -1;
        check(nbg_add_bodies(ctx_.get(), &soa, 1, &id));
        b.Id = id;
        remember(b);
        return id;
    }

    /* ModBody (body_collection.go:154-191): matches by class, name or id. */
    ModBodyResult ModBody(int64_t id, const std::string &name, const std::string &cls,
                          const std::vector<std::string> &mods)
    {
        std::vector<Body> arr = GetArray();
        std::vector<nbg_edit> edits;
        int found = 0;
        for (const Body &b : arr) {
            const Names &nm = names_[b.Id];
            if ((!cls.empty() && cls == nm.cls) || (!name.empty() && name == nm.name) || id == b.Id) {
                found++;
                edits.push_back(EditFromMods(b.Id, mods, b));
                Body h = b;
                h.ApplyMods(mods);
                if (h.Color != b.Color) names_[b.Id].color = h.Color;
            }
        }
        if (found == 0) return NoMatch;
        std::vector<int32_t> res(edits.size());
        check(nbg_apply_edits(ctx_.get(), edits.data(), (int64_t)edits.size(), res.data()));
        return ModAll; /* ApplyMods always reports success */
    }

    /* GetBody (body_collection.go:111-135): first body with the name (if
     * given) or the id; nullptr if none. */
    std::unique_ptr<Body> GetBody(int64_t id, const std::string &name)
    {
        for (const Body &b : GetArray())
            if ((!name.empty() && name == names_[b.Id].name) || id == b.Id) return std::unique_ptr<Body>(new Body(b));
        return nullptr;
    }

    int64_t Count()
    {
        int64_t n = 0;
        check(nbg_count(ctx_.get(), &n));
        return n;
    }

    /* a copy of the body array, in array order */
    std::vector<Body> GetArray()
    {
        int64_t n = Count();
        SoaBuffers s;
        s.resize((size_t)n);
        nbg_soa soa = s.soa();
        check(nbg_get_state(ctx_.get(), &soa, n, &n));
        std::vector<Body> out((size_t)n);
        for (size_t k = 0; k < (size_t)n; k++) {
            out[k] = s.get(k);
            auto it = names_.find(out[k].Id);
            if (it != names_.end()) {
                out[k].Name = it->second.name;
                out[k].Class = it->second.cls;
                out[k].Color = it->second.color;
            }
        }
        return out;
    }

    void check(int rc) const
    {
        if (rc != NBG_OK) throw Error(rc, nbg_last_error(ctx_.get()));
    }

  private:
    struct Names {
        std::string name, cls;
        BodyColor color = Random;
    };
    struct Del {
        void operator()(nbg_ctx *c) const { nbg_destroy(c); }
    };
    void remember(const Body &b) { names_[b.Id] = Names{b.Name, b.Class, b.Color}; }
    std::unique_ptr<nbg_ctx, Del> ctx_;
    std::map<int64_t, Names> names_;
};

/* ComputationRunner (computation-runner.go:24-326) over the GPU cycle. */
class ComputationRunner {
  public:
    /* NewComputationRunner(workerCnt, timeScaling, barnesHut, rqh, bc):
     * barnesHut selects the octree force pass (with the tree built every
     * cycle, which the reference's BuildTree omits). */
    ComputationRunner(int workerCnt, double timeScaling, bool barnesHut, BodyCollection &bc)
        : bc_(bc), workers_(workerCnt), dt_(timeScaling)
    {
        bc_.check(nbg_set_option(bc_.ctx(), NBG_OPT_BARNES_HUT, barnesHut ? 1 : 0));
    }

    /* setters take effect at the start of the next cycle (1-slot channels) */
    void SetTimeScaling(double dt) { pending_dt_ = dt; has_dt_ = true; }
    void SetCoefficientOfRestitution(double R) { pending_R_ = R; has_R_ = true; }
    void SetWorkers(int n) { workers_ = n; } /* the GPU grid replaces the pool */
    void RemoveBodies(int64_t n) { pending_del_ = n; has_del_ = true; }
    double TimeScaling() const { return dt_; }
    double CoefficientOfRestitution() const { return R_; }
    int WorkerCount() const { return workers_; }

    /* runOneComputation (computation-runner.go:267-326): setters, deletes,
     * then one cycle.  Returns the renderables of the cycle's Update. */
    std::vector<nbg_renderable> RunOneComputation()
    {
        if (has_dt_) { dt_ = pending_dt_; has_dt_ = false; }
        if (has_R_) { R_ = pending_R_; has_R_ = false; }
        if (has_del_) {
            has_del_ = false;
            int64_t removed = 0;
            bc_.check(nbg_remove_bodies(bc_.ctx(), pending_del_, &removed));
        }
        /* fragments take ids from the same counter as NextId */
        int64_t dev_next = 0;
        bc_.check(nbg_get_next_id(bc_.ctx(), &dev_next));
        const int64_t host_next = next_id_counter().load();
        if (host_next > dev_next) bc_.check(nbg_set_next_id(bc_.ctx(), host_next));
        nbg_step_info info{};
        bc_.check(nbg_step(bc_.ctx(), dt_, R_, 1, &info));
        AdvanceNextId(info.next_id);
        int64_t n = 0;
        bc_.check(nbg_get_renderables(bc_.ctx(), nullptr, 0, &n));
        std::vector<nbg_renderable> out((size_t)n);
        bc_.check(nbg_get_renderables(bc_.ctx(), out.data(), n, &n));
        computations_++;
        return out;
    }
    uint64_t Computations() const { return computations_; }

    /* A checkpoint of the whole simulation: the library snapshot
     * (nbg_save_state: every body field, private ones included, the id
     * counter, the fragment generator's cycle key, staged adds, options)
     * after a small runner header (its dt, R and computation count).
     * LoadSnapshot, in this runner or another, resumes the run bit for bit.
     * No counterpart in the reference, whose CSV (FromCsv / ToCsv) keeps only
     * the public fields. */
    std::vector<uint8_t> SaveSnapshot() const
    {
        int64_t size = 0;
        bc_.check(nbg_save_state(bc_.ctx(), nullptr, 0, &size));
        std::vector<uint8_t> out(kRunnerHeader + (size_t)size);
        std::memcpy(out.data(), "NBGRUN01", 8);
        std::memcpy(out.data() + 8, &dt_, 8);
        std::memcpy(out.data() + 16, &R_, 8);
        std::memcpy(out.data() + 24, &computations_, 8);
        bc_.check(nbg_save_state(bc_.ctx(), out.data() + kRunnerHeader, size, &size));
        return out;
    }
    void LoadSnapshot(const std::vector<uint8_t> &snap)
    {
        if (snap.size() < kRunnerHeader || std::memcmp(snap.data(), "NBGRUN01", 8) != 0)
            throw Error(NBG_E_ARG, "not a runner snapshot");
        bc_.check(nbg_load_state(bc_.ctx(), snap.data() + kRunnerHeader, (int64_t)(snap.size() - kRunnerHeader)));
        std::memcpy(&dt_, snap.data() + 8, 8);
        std::memcpy(&R_, snap.data() + 16, 8);
        std::memcpy(&computations_, snap.data() + 24, 8);
        has_dt_ = has_R_ = has_del_ = false;
        int64_t dev_next = 0;
        bc_.check(nbg_get_next_id(bc_.ctx(), &dev_next));
        AdvanceNextId(dev_next);
    }

  private:
    static constexpr size_t kRunnerHeader = 32;
    BodyCollection &bc_;
    int workers_;
    double dt_, R_ = 1.0;
    double pending_dt_ = 0, pending_R_ = 0;
    int64_t pending_del_ = 0;
    bool has_dt_ = false, has_R_ = false, has_del_ = false;
    uint64_t computations_ = 0;
};

} // namespace nbodygo

#endif

/*
 * The reference's own Go tests of the body collection, the body and the
 * runner, restated against the C++ mirror (include/nbodygo.hpp) over
 * libnbgpu.so:
 *
 *   TestMod                      cmd/body/body_test.go:9-47
 *   TestInitSize                 cmd/body/body_collection_test.go:61-67
 *   TestRemove                   cmd/body/body_collection_test.go:73-89
 *   TestGetByID / ByName         cmd/body/body_collection_test.go:94-148
 *   TestModByID / NoMatch /      cmd/body/body_collection_test.go:154-262
 *     ByName / ByClass
 *   TestAdds                     cmd/body/body_collection_test.go:268-282
 *   TestRunnerSetters            cmd/runner/computation-runner_test.go:10-31
 *
 * and FromCsv (cmd/sim/fromcsv.go:46-131) on the format its header
 * documents, with the ToCsv snapshot read back bit for bit.
 *
 * The bodies are those of createTestBody (body_collection_test.go:26-54):
 * every field equal to the id, Name = Class = string(rune(id)).  The Go
 * tests call Cycle/ProcessMods alone; here the whole cycle runs, so bodies
 * that must not collide are given collision=none (no events, body.go:175-178),
 * and body 0, whose mass is 0, leaves the collection too: Update computes
 * v += (dt * 0) / 0 = NaN, and a NaN position clears Exists (body.go:114-139).
 *
 * Usage: test_mirror host   - parsing and ApplyMods, no GPU
 *        test_mirror gpu    - everything, on device 0
 * Prints one line per test and exits non-zero if any failed.
 */
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "nbodygo.hpp"

using namespace nbodygo;

static int g_fail = 0;
#define CHECK(cond, what)                                                                                        \
    do {                                                                                                         \
        if (!(cond)) {                                                                                           \
            std::printf("FAIL %s: %s (line %d)\n", cur_test, what, __LINE__);                                    \
            g_fail = 1;                                                                                          \
            return;                                                                                              \
        }                                                                                                        \
    } while (0)
static const char *cur_test = "";

/* Go's string(int): the UTF-8 encoding of the code point */
static std::string go_string(int cp)
{
    std::string s;
    if (cp < 0x80) s += (char)cp;
    else if (cp < 0x800) {
        s += (char)(0xC0 | (cp >> 6));
        s += (char)(0x80 | (cp & 0x3F));
    } else if (cp < 0x10000) {
        s += (char)(0xE0 | (cp >> 12));
        s += (char)(0x80 | ((cp >> 6) & 0x3F));
        s += (char)(0x80 | (cp & 0x3F));
    } else {
        s += (char)(0xF0 | (cp >> 18));
        s += (char)(0x80 | ((cp >> 12) & 0x3F));
        s += (char)(0x80 | ((cp >> 6) & 0x3F));
        s += (char)(0x80 | (cp & 0x3F));
    }
    return s;
}

static Body createTestBody(int id, CollisionBehavior beh = Elastic)
{
    Body b;
    b.Id = id;
    b.Name = b.Class = go_string(id);
    b.X = b.Y = b.Z = b.Vx = b.Vy = b.Vz = b.Radius = b.Mass = b.FragFactor = b.FragStep = (double)id;
    b.Behavior = beh;
    b.Color = Red;
    return b;
}

static std::vector<Body> createTestBodies(int cnt, CollisionBehavior beh = Elastic)
{
    std::vector<Body> v;
    v.reserve(cnt);
    for (int i = 0; i < cnt; i++) v.push_back(createTestBody(i, beh));
    return v;
}

static void TestMod()
{
    cur_test = "TestMod";
    Body b = createTestBody(1);
    b.ApplyMods({"x=41", "y=42", "z=43", "vx=44", "vy=45", "vz=46", "mass=47", "radius=48", "frag-factor=49",
                 "frag-step=50", "collision=subsume", "color=green", "telemetry=true", "exists=false"});
    CHECK(b.X == 41 && b.Y == 42 && b.Z == 43 && b.Vx == 44 && b.Vy == 45 && b.Vz == 46, "position/velocity");
    CHECK(b.Mass == 47 && b.Radius == 48 && b.FragFactor == 49 && b.FragStep == 50, "mass/radius/frag");
    CHECK(b.Behavior == Subsume && b.Color == Green && b.WithTelemetry && !b.Exists, "enums/bools");
    std::printf("ok   %s\n", cur_test);
}

static void TestParse()
{
    cur_test = "TestParse";
    CHECK(ParseCollisionBehavior("FRAGMENT") == Fragment && ParseCollisionBehavior("bogus") == Elastic,
          "ParseCollisionBehavior");
    CHECK(ParseBoolean("Yes") && ParseBoolean("1") && !ParseBoolean("on"), "ParseBoolean");
    CHECK(ParseBodyColor("LightGray") == Lightgray && ParseBodyColor("teal") == Random, "ParseBodyColor");
    CHECK(SafeParseFloat("2.5e3", 1) == 2500 && SafeParseFloat("12abc", 7) == 7 && SafeParseFloat("", 3) == 3 &&
              SafeParseFloat(" 1", 4) == 4,
          "SafeParseFloat");
    Body b = createTestBody(3);
    b.ApplyMods({"x=1=2", "mass=heavy", "nosuch=1", "RADIUS=9"});
    CHECK(b.X == 3 && b.Mass == 3 && b.Radius == 9, "malformed mods are ignored");
    Body sun = createTestBody(4);
    sun.IsSun = true;
    sun.Color = White;
    sun.ApplyMods({"color=blue"});
    CHECK(sun.Color == White, "suns keep their colour");
    std::printf("ok   %s\n", cur_test);
}

static void TestFromCsv()
{
    cur_test = "TestFromCsv";
    const std::string path = "test_mirror_in.csv";
    {
        std::ofstream o(path);
        o << "# a comment\n"
          << "100,100,100,100,100,100,10,.5,,,blue\n"   /* empty is_sun does not parse: skipped */
          << "1,1,1,1,1,1,10000,10,true,elastic\n"      /* a sun */
          << "\n"
          << " 2 , 3 ,4,5,6,7,8,9,F,SUBSUME,Green,1.5,2.5\n"
          << "1,2,3,4,5,6,7\n"                         /* radius missing: skipped */
          << "1,2,3,4,5,6,7,x\n"                       /* radius does not parse: skipped */
          << "\"-1e3\",0,0,0,0,0,1,1,0,bogus,teal\n"    /* quoted field; unknown names take defaults */
          << "9,9,9,9,9,9,9,9\n";
    }
    const int64_t id0 = next_id_counter().load();
    std::vector<Body> b = FromCsv(path, 1000, Fragment, Cyan);
    CHECK(b.size() == 4, "record count");
    CHECK(b[0].IsSun && b[0].X == 1 && b[0].Mass == 10000 && b[0].Radius == 10 && b[0].Behavior == Elastic &&
              b[0].Color == Cyan && b[0].intensity == 100,
          "sun record");
    CHECK(!b[1].IsSun && b[1].X == 2 && b[1].Y == 3 && b[1].Vz == 7 && b[1].Behavior == Subsume &&
              b[1].Color == Green && b[1].FragFactor == 1.5 && b[1].FragStep == 2.5,
          "full record");
    CHECK(b[2].X == -1e3 && b[2].Behavior == Elastic && b[2].Color == Random, "quoted record, unknown names");
    CHECK(b[3].Behavior == Fragment && b[3].Color == Cyan && b[3].FragFactor == 0, "defaults");
    CHECK(b[0].Id == id0 && b[3].Id == id0 + 3, "ids from NextId");
    CHECK(FromCsv(path, 2, Elastic, Random).size() == 2, "bodyCount limit");
    CHECK(FromCsv("no_such_file.csv", 10, Elastic, Random).empty(), "missing file");
    /* snapshot round trip */
    b[1].X = 0.1 + 0.2;
    b[1].Vy = -1.0 / 3.0;
    CHECK(ToCsv("test_mirror_snap.csv", b), "write snapshot");
    std::vector<Body> r = FromCsv("test_mirror_snap.csv", 1000, None, Random);
    CHECK(r.size() == b.size(), "snapshot count");
    for (size_t k = 0; k < r.size(); k++)
        CHECK(r[k].X == b[k].X && r[k].Y == b[k].Y && r[k].Z == b[k].Z && r[k].Vx == b[k].Vx && r[k].Vy == b[k].Vy &&
                  r[k].Vz == b[k].Vz && r[k].Mass == b[k].Mass && r[k].Radius == b[k].Radius &&
                  r[k].IsSun == b[k].IsSun && r[k].Behavior == b[k].Behavior && r[k].Color == b[k].Color &&
                  r[k].FragFactor == b[k].FragFactor && r[k].FragStep == b[k].FragStep,
              "snapshot values");
    {
        std::ofstream o("test_mirror_bad.csv");
        o << "1,2,3,4,5,6,7,8x\"y\n";
    }
    bool threw = false;
    try {
        FromCsv("test_mirror_bad.csv", 10, Elastic, Random);
    } catch (const Error &) {
        threw = true;
    }
    CHECK(threw, "bare quote is an error");
    std::remove(path.c_str());
    std::remove("test_mirror_snap.csv");
    std::remove("test_mirror_bad.csv");
    std::printf("ok   %s\n", cur_test);
}

static void TestInitSize()
{
    cur_test = "TestInitSize";
    const int cnt = 1000000;
    BodyCollection bc(createTestBodies(cnt));
    CHECK(bc.Count() == cnt, "Incorrect body count");
    std::printf("ok   %s\n", cur_test);
}

static void TestRemove()
{
    cur_test = "TestRemove";
    const int cnt = 1000, idToDelete = 10;
    BodyCollection bc(createTestBodies(cnt, None));
    CHECK(bc.ModBody(idToDelete, "", "", {"exists=false"}) == ModAll, "mod");
    ComputationRunner cr(1, 1e-9, false, bc);
    cr.RunOneComputation();
    CHECK(bc.Count() == cnt - 2, "Body was not removed (body 0 leaves by the NaN rule)");
    for (const Body &b : bc.GetArray()) CHECK(b.Id != idToDelete && b.Id != 0, "Body should have been removed");
    std::printf("ok   %s\n", cur_test);
}

static void TestGetByID()
{
    cur_test = "TestGetByID";
    BodyCollection bc(createTestBodies(1000));
    auto b = bc.GetBody(10, "");
    CHECK(b != nullptr, "Got nil body");
    CHECK(b->Id == 10, "Got wrong body");
    std::printf("ok   %s\n", cur_test);
}

static void TestGetByName()
{
    cur_test = "TestGetByName";
    BodyCollection bc(createTestBodies(2000));
    auto b = bc.GetBody(-1, go_string(1999));
    CHECK(b != nullptr, "Got nil body");
    CHECK(b->Id == 1999, "Got wrong body");
    std::printf("ok   %s\n", cur_test);
}

static void mod_test(const char *name, int id, const std::string &nm, const std::string &cls, int idToGet,
                     ModBodyResult want)
{
    cur_test = name;
    BodyCollection bc(createTestBodies(1000));
    ModBodyResult r = bc.ModBody(id, nm, cls, {"color=blue"});
    CHECK(r == want, "Mod body failed");
    if (want == ModAll) {
        std::vector<Body> arr = bc.GetArray();
        CHECK(arr[idToGet].Color == Blue, "Body modification failed");
    }
    std::printf("ok   %s\n", cur_test);
}

static void TestModPhysical()
{
    cur_test = "TestModPhysical";
    BodyCollection bc(createTestBodies(100));
    CHECK(bc.ModBody(7, "", "", {"x=-5", "mass=123.5", "collision=fragment", "telemetry=yes"}) == ModAll, "mod");
    auto b = bc.GetBody(7, "");
    CHECK(b && b->X == -5 && b->Mass == 123.5 && b->Behavior == Fragment && b->WithTelemetry && b->Y == 7,
          "numeric mods reach the device copy");
    std::printf("ok   %s\n", cur_test);
}

static void TestAdds()
{
    cur_test = "TestAdds";
    const int cnt = 500, idToAdd = 600;
    BodyCollection bc(createTestBodies(cnt, None));
    bc.EnqueueAdd(createTestBody(idToAdd, None));
    ComputationRunner cr(1, 1e-9, false, bc);
    cr.RunOneComputation();
    bool found = false;
    for (const Body &b : bc.GetArray()) found |= b.Id == idToAdd;
    CHECK(found, "Body was not added");
    CHECK(bc.Count() == cnt, "count after add (body 0 leaves by the NaN rule)");
    std::printf("ok   %s\n", cur_test);
}

static void TestRunnerSetters()
{
    cur_test = "TestRunnerSetters";
    BodyCollection bc(std::vector<Body>{});
    ComputationRunner cr(1, 1, true, bc); /* Barnes-Hut, as the reference test */
    cr.SetCoefficientOfRestitution(5);
    cr.SetTimeScaling(5);
    cr.SetWorkers(5);
    cr.RunOneComputation(); /* the setters are picked up at the start of a cycle */
    CHECK(cr.CoefficientOfRestitution() == 5 && cr.TimeScaling() == 5 && cr.WorkerCount() == 5, "Setters failed");
    std::printf("ok   %s\n", cur_test);
}

static void TestRunnerBarnesHut()
{
    cur_test = "TestRunnerBarnesHut";
    /* with the tree built, Barnes-Hut applies gravity (the reference's
     * BuildTree alone would leave every force at zero) */
    std::vector<Body> v;
    for (int k = 0; k < 64; k++)
        v.push_back(NewBody(k, (k % 4) * 10.0, (k / 4 % 4) * 10.0, (k / 16) * 10.0, 0, 0, 0, 1e12, 0.1, Elastic, Random,
                            0, 0, false, "", "", false));
    BodyCollection bc(v);
    ComputationRunner cr(4, 0.01, true, bc);
    cr.RunOneComputation();
    std::vector<Body> arr = bc.GetArray();
    CHECK(arr.size() == 64, "count");
    CHECK(arr[0].Vx > 0 && arr[0].Vy > 0 && arr[0].Vz > 0, "the corner body falls inward");
    CHECK(arr[63].Vx < 0 && arr[63].Vy < 0 && arr[63].Vz < 0, "the far corner too");
    std::printf("ok   %s\n", cur_test);
}

static void TestRunnerCycle()
{
    cur_test = "TestRunnerCycle";
    /* two bodies at rest attract: after one cycle each moved toward the other */
    std::vector<Body> v;
    v.push_back(NewBody(1, -1, 0, 0, 0, 0, 0, 1e10, 0.1, None, Random, 0, 0, false, "a", "", false));
    v.push_back(NewBody(2, 1, 0, 0, 0, 0, 0, 1e10, 0.1, None, Random, 0, 0, false, "b", "", false));
    BodyCollection bc(v);
    ComputationRunner cr(4, 0.5, false, bc);
    std::vector<nbg_renderable> rend = cr.RunOneComputation();
    CHECK(rend.size() == 2, "renderables");
    std::vector<Body> arr = bc.GetArray();
    CHECK(arr.size() == 2 && arr[0].X > -1 && arr[1].X < 1 && arr[0].Vx > 0 && arr[1].Vx < 0, "attraction");
    CHECK(arr[0].X == -arr[1].X && arr[0].Vx == -arr[1].Vx, "symmetry");
    cr.RemoveBodies(-1);
    cr.RunOneComputation();
    CHECK(bc.Count() == 0, "RemoveBodies(-1) empties the collection");
    std::printf("ok   %s\n", cur_test);
}

/* Not a reference test: a checkpoint taken mid-run and resumed in a fresh
 * collection and runner repeats the uninterrupted run bit for bit. */
static void TestRunnerSnapshot()
{
    cur_test = "TestRunnerSnapshot";
    auto cluster = []() {
        std::vector<Body> v;
        for (int k = 0; k < 64; k++) {
            const double a = 0.7 * k;
            v.push_back(NewBody(k + 1, 8 * std::cos(a), 8 * std::sin(a), 0.3 * (k % 5), -std::sin(a), std::cos(a),
                                0, 1e11 * (1 + k % 3), 0.6 + 0.2 * (k % 4), k % 2 ? Elastic : Subsume, Random, 0, 0, false,
                                "b" + std::to_string(k), "", false));
        }
        return v;
    };
    BodyCollection ba(cluster());
    ComputationRunner ra(4, 0.05, false, ba);
    ra.SetCoefficientOfRestitution(0.8);
    for (int c = 0; c < 10; c++) ra.RunOneComputation();
    const std::vector<uint8_t> snap = ra.SaveSnapshot();
    for (int c = 0; c < 10; c++) ra.RunOneComputation();
    BodyCollection bb(std::vector<Body>{});
    ComputationRunner rb(4, 1.0, false, bb);
    rb.LoadSnapshot(snap);
    CHECK(rb.TimeScaling() == 0.05 && rb.CoefficientOfRestitution() == 0.8 && rb.Computations() == 10,
          "runner settings restored");
    for (int c = 0; c < 10; c++) rb.RunOneComputation();
    const std::vector<Body> x = ba.GetArray(), y = bb.GetArray();
    CHECK(x.size() == y.size() && x.size() < 64, "same bodies, some merged");
    for (size_t k = 0; k < x.size(); k++)
        CHECK(x[k].Id == y[k].Id && x[k].X == y[k].X && x[k].Y == y[k].Y && x[k].Z == y[k].Z &&
                  x[k].Vx == y[k].Vx && x[k].Vy == y[k].Vy && x[k].Vz == y[k].Vz && x[k].Mass == y[k].Mass,
              "bit-identical state after the resume");
    std::printf("ok   %s\n", cur_test);
}

int main(int argc, char **argv)
{
    const std::string mode = argc > 1 ? argv[1] : "host";
    TestMod();
    TestParse();
    TestFromCsv();
    if (mode == "gpu" && !g_fail) {
        try {
            TestInitSize();
            TestRemove();
            TestGetByID();
            TestGetByName();
            mod_test("TestModByID", 10, "", "", 10, ModAll);
            mod_test("TestModByIDNoMatch", 2000, "", "", 0, NoMatch);
            mod_test("TestModByName", -1, go_string(10), "", 10, ModAll);
            mod_test("TestModByClass", -1, "", go_string(10), 10, ModAll);
            TestModPhysical();
            TestAdds();
            TestRunnerSetters();
            TestRunnerBarnesHut();
            TestRunnerCycle();
            TestRunnerSnapshot();
        } catch (const Error &e) {
            std::printf("FAIL %s: nbg status %d: %s\n", cur_test, e.code, e.what());
            g_fail = 1;
        }
    }
    std::printf(g_fail ? "FAILED\n" : "PASSED\n");
    return g_fail;
}

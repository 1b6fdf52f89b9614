"""Generates the golden fixtures of tests/golden/*.json.

A second, independent restatement of the reference's direct-sum compute
cycle, written as plain Python loops over body records (Python floats are
IEEE doubles and Python never fuses a multiply-add, like Go on amd64):

  Compute          cmd/body/body.go:148-187 (calcForceFrom :214-225,
                   Collided :192-208, event creation :172-186)
  fragment         cmd/body/fragcalc.go:94-117
  ProcessMods      cmd/body/body_collection.go:212-233 (newest event first)
  ResolveCollision cmd/body/body.go:248-264, collisioncalc.go:26-186,
                   fragcalc.go:24-85
  ResolveSubsume   cmd/body/body.go:228-244
  Update           cmd/body/body.go:114-139
  Cycle            cmd/body/body_collection.go:253-296

It shares two things with the C oracle by design: the FP64 elementary
functions (nbg_math.h, called through the oracle library's test hook, since
Go's own math package cannot run here) and the seeded fragment-position
generator (restated below).  Everything else is written from the Go source
independently of oracle/nbg_oracle.c.

    python tests/golden/make_golden.py      # rewrites the fixtures
"""
import json
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import math_eval  # noqa: E402

G = 6.673e-11
NONE, SUBSUME, ELASTIC, FRAGMENT = 0, 1, 2, 3
MASK = (1 << 64) - 1


def acos(x): return math_eval(4, x)
def asin(x): return math_eval(3, x)
def atan2(y, x): return math_eval(6, y, x)
def sin(x): return math_eval(0, x)
def cos(x): return math_eval(1, x)
def tan(x): return math_eval(2, x)


def go_min(x, y):
    if x != x or y != y:
        return math.nan
    if x == 0.0 and y == 0.0:
        return x if math.copysign(1, x) < 0 else y
    return x if x < y else y


def _mix(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
    return z ^ (z >> 31)


def frag_point(seed, parent, cycle, cnt, cx, cy, cz, radius):
    k = _mix((seed + 0x9E3779B97F4A7C15) & MASK)
    k = _mix(k ^ ((parent * 0xD1B54A32D192ED03) & MASK))
    k = _mix(k ^ ((cycle * 0xAEF17502108EF2D9 + 0x632BE59BD9B4E019) & MASK))

    def u(ctr):
        return (_mix((k + (ctr + 1) * 0x9E3779B97F4A7C15) & MASK) >> 11) * 2.0 ** -53
    x = y = z = 0.0
    for a in range(85):
        base = cnt * 256 + 3 * a
        x, y, z = u(base) * 2 - 1, u(base + 1) * 2 - 1, u(base + 2) * 2 - 1
        d = x * x + y * y + z * z
        if not d > 1:
            break
    else:
        x = y = z = 0.0
    return (x * radius) + cx, (y * radius) + cy, (z * radius) + cz


class Body:
    FIELDS = ("id", "x", "y", "z", "vx", "vy", "vz", "radius", "mass", "frag_factor", "frag_step", "collision",
              "exists", "is_sun", "pinned", "telemetry", "r", "fragmenting", "collided", "fx", "fy", "fz",
              "fr_radius", "fr_new_radius", "fr_mass", "fr_fragments", "fr_cx", "fr_cy", "fr_cz")

    def __init__(self, **kw):
        self.id = 0
        self.x = self.y = self.z = self.vx = self.vy = self.vz = 0.0
        self.radius = self.mass = self.frag_factor = self.frag_step = 0.0
        self.collision = ELASTIC
        self.exists, self.is_sun, self.pinned, self.telemetry = True, False, False, False
        self.r = 1.0
        self.fragmenting = self.collided = False
        self.fx = self.fy = self.fz = 0.0
        self.fr_radius = self.fr_new_radius = self.fr_mass = 0.0
        self.fr_fragments = 0
        self.fr_cx = self.fr_cy = self.fr_cz = 0.0
        for k, v in kw.items():
            setattr(self, k, v)


class Sim:
    def __init__(self, bodies, seed, next_id):
        self.arr = bodies
        self.events = []  # arrival order: (kind, b1, b2)
        self.seed = seed
        self.cycle = 0
        self.next_id = next_id
        self.handled = []

    # body.go:214-225
    @staticmethod
    def calc_force_from(b, o):
        dx = o.x - b.x
        dy = o.y - b.y
        dz = o.z - b.z
        dist = math.sqrt(dx * dx + dy * dy + dz * dz)
        if b.collided or dist > b.radius + o.radius:
            force = G * b.mass * o.mass / (dist * dist)
            b.fx += force * dx / dist
            b.fy += force * dy / dist
            b.fz += force * dz / dist

    # body.go:192-208
    @staticmethod
    def collided_with(b, o):
        if b.collided:
            return False, 0.0
        dx = o.x - b.x
        dy = o.y - b.y
        dz = o.z - b.z
        dist = math.sqrt(dx * dx + dy * dy + dz * dz)
        if dist > b.radius + o.radius:
            return False, 0.0
        elif dist <= b.radius + o.radius:
            return True, dist
        return False, 0.0

    def fragment(self, b, pending_exists_false):
        cnt = 0
        while b.fr_fragments > 0:
            b.fr_fragments -= 1
            px, py, pz = frag_point(self.seed, b.id, self.cycle, cnt, b.fr_cx, b.fr_cy, b.fr_cz, b.fr_radius * .9)
            f = Body(id=None, x=px, y=py, z=pz, vx=b.vx, vy=b.vy, vz=b.vz, mass=b.fr_mass, radius=b.fr_new_radius,
                     frag_factor=0.0, frag_step=0.0, collision=ELASTIC, r=0.0)
            self.events.append(("add", f, None))
            cnt += 1
            if cnt > 100:
                break
        if b.fr_fragments <= 0:
            pending_exists_false.append(b)

    def compute(self):
        gone = []
        for b in self.arr:
            if not b.exists:
                continue
            if b.fragmenting:
                self.fragment(b, gone)
                continue
            b.fx = b.fy = b.fz = 0.0
            for o in self.arr:
                if not o.exists or b.fragmenting:
                    continue
                if b is not o and o.exists and not o.fragmenting:
                    self.calc_force_from(b, o)
            for o in self.arr:
                hit, dist = self.collided_with(b, o)
                if not hit:
                    continue
                if b.collision in (ELASTIC, FRAGMENT) and o.collision in (ELASTIC, FRAGMENT):
                    self.events.append(("collision", b, o))
                elif b.collision == SUBSUME or o.collision == SUBSUME:
                    if b.radius > o.radius and dist <= b.radius:
                        self.events.append(("subsume", b, o))
                    elif o.radius > b.radius and dist <= o.radius:
                        self.events.append(("subsume", o, b))
        for b in gone:
            b.exists = False
        for kind, b1, _ in self.events:
            if kind == "add" and b1.id is None:
                b1.id = self.next_id
                self.next_id += 1

    # collisioncalc.go:42-186
    @staticmethod
    def elastic(b, o):
        m1, m2, r1, r2 = b.mass, o.mass, b.radius, o.radius
        x1, y1, z1, x2, y2, z2 = b.x, b.y, b.z, o.x, o.y, o.z
        vx1, vy1, vz1, vx2, vy2, vz2 = b.vx, b.vy, b.vz, o.vx, o.vy, o.vz
        r12 = r1 + r2
        m21 = m2 / m1
        x21, y21, z21 = x2 - x1, y2 - y1, z2 - z1
        vx21, vy21, vz21 = vx2 - vx1, vy2 - vy1, vz2 - vz1
        vx_cm = (m1 * vx1 + m2 * vx2) / (m1 + m2)
        vy_cm = (m1 * vy1 + m2 * vy2) / (m1 + m2)
        vz_cm = (m1 * vz1 + m2 * vz2) / (m1 + m2)
        d = math.sqrt(x21 * x21 + y21 * y21 + z21 * z21)
        v = math.sqrt(vx21 * vx21 + vy21 * vy21 + vz21 * vz21)
        if v == 0:
            return None
        x2, y2, z2 = x21, y21, z21
        vx1, vy1, vz1 = -vx21, -vy21, -vz21
        theta2 = acos(z2 / d) if d != 0 else acos(math.nan)
        phi2 = 0.0 if (x2 == 0 and y2 == 0) else atan2(y2, x2)
        st, ct, sp, cp = sin(theta2), cos(theta2), sin(phi2), cos(phi2)
        vx1r = ct * cp * vx1 + ct * sp * vy1 - st * vz1
        vy1r = cp * vy1 - sp * vx1
        vz1r = st * cp * vx1 + st * sp * vy1 + ct * vz1
        fvz1r = vz1r / v
        if fvz1r > 1:
            fvz1r = 1.0
        elif fvz1r < -1:
            fvz1r = -1.0
        thetav = acos(fvz1r)
        phiv = 0.0 if (vx1r == 0 and vy1r == 0) else atan2(vy1r, vx1r)
        dr = d * sin(thetav) / r12
        if thetav > math.pi / 2 or abs(dr) > 1:
            return None
        alpha = asin(-dr)
        beta = phiv
        sbeta, cbeta = sin(beta), cos(beta)
        a = tan(thetav + alpha)
        dvz2 = 2 * (vz1r + a * (cbeta * vx1r + sbeta * vy1r)) / ((1 + a * a) * (1 + m21))
        vz2r = dvz2
        vx2r = a * cbeta * dvz2
        vy2r = a * sbeta * dvz2
        vz1r = vz1r - m21 * vz2r
        vx1r = vx1r - m21 * vx2r
        vy1r = vy1r - m21 * vy2r
        return dict(
            vx1=ct * cp * vx1r - sp * vy1r + st * cp * vz1r + vx2,
            vy1=ct * sp * vx1r + cp * vy1r + st * sp * vz1r + vy2,
            vz1=ct * vz1r - st * vx1r + vz2,
            vx2=ct * cp * vx2r - sp * vy2r + st * cp * vz2r + vx2,
            vy2=ct * sp * vx2r + cp * vy2r + st * sp * vz2r + vy2,
            vz2=ct * vz2r - st * vx2r + vz2,
            vx_cm=vx_cm, vy_cm=vy_cm, vz_cm=vz_cm)

    @staticmethod
    def initiate_fragmentation(b, frag_factor):
        frag_delta = 10.0 if b.frag_factor > 10 else frag_factor - b.frag_factor
        fragments = go_min(frag_delta * b.frag_step, 2000.0)
        if fragments <= 1:
            b.collision = FRAGMENT
            return
        b.fragmenting = True
        b.fr_radius = b.radius
        b.fr_new_radius = 1.0  # math.Pow(x, 1/3) with Go's integer 1/3 == 0
        b.fr_mass = b.mass / fragments
        b.fr_fragments = 0 if fragments != fragments else int(fragments)
        b.fr_cx, b.fr_cy, b.fr_cz = b.x, b.y, b.z

    def resolve_collision(self, b, o):
        if not b.exists or not o.exists:
            return
        if b.collision == ELASTIC and o.collision in (ELASTIC, FRAGMENT):
            r = self.elastic(b, o)
            if r is None:
                return
            # shouldFragment, fragcalc.go:24-49
            frag, tf, of = False, 0.0, 0.0
            if b.collision == FRAGMENT or o.collision == FRAGMENT:
                v_this = b.vx + b.vy + b.vz
                dv_this = (abs(b.vx - ((r["vx1"] - r["vx_cm"]) * b.r + r["vx_cm"])) +
                           abs(b.vy - ((r["vy1"] - r["vy_cm"]) * b.r + r["vy_cm"])) +
                           abs(b.vz - ((r["vz1"] - r["vz_cm"]) * b.r + r["vz_cm"])))
                this_factor = dv_this / abs(v_this) if v_this != 0 else (math.inf if dv_this > 0 else math.nan)
                v_other = o.vx + o.vy + o.vz
                dv_other = (abs(o.vx - ((r["vx2"] - r["vx_cm"]) * b.r + r["vx_cm"])) +
                            abs(o.vy - ((r["vy2"] - r["vy_cm"]) * b.r + r["vy_cm"])) +
                            abs(o.vz - ((r["vz2"] - r["vz_cm"]) * b.r + r["vz_cm"])))
                other_factor = dv_other / abs(v_other) if v_other != 0 else (math.inf if dv_other > 0 else math.nan)
                if (b.collision == FRAGMENT and this_factor > b.frag_factor) or \
                        (o.collision == FRAGMENT and other_factor > o.frag_factor):
                    frag, tf, of = True, this_factor, other_factor
            if frag:
                if b.collision == FRAGMENT and tf > b.frag_factor:
                    self.initiate_fragmentation(b, tf)
                if o.collision == FRAGMENT and of > o.frag_factor:
                    self.initiate_fragmentation(o, of)
                return
            b.vx = (r["vx1"] - r["vx_cm"]) * b.r + r["vx_cm"]
            b.vy = (r["vy1"] - r["vy_cm"]) * b.r + r["vy_cm"]
            b.vz = (r["vz1"] - r["vz_cm"]) * b.r + r["vz_cm"]
            o.vx = (r["vx2"] - r["vx_cm"]) * b.r + r["vx_cm"]
            o.vy = (r["vy2"] - r["vy_cm"]) * b.r + r["vy_cm"]
            o.vz = (r["vz2"] - r["vz_cm"]) * b.r + r["vz_cm"]
            b.collided = o.collided = True

    @staticmethod
    def resolve_subsume(b, o):
        this_mass, other_mass = b.mass, o.mass
        b.mass = this_mass + other_mass
        o.mass = 0.0
        o.exists = False

    def process_mods(self):
        self.handled = []
        for kind, b1, b2 in reversed(self.events):
            if kind == "add":
                continue
            if b1 is not b2:
                self.handled.append((b1.id, b2.id, 0 if kind == "collision" else 1))
            if kind == "collision":
                self.resolve_collision(b1, b2)
            else:
                self.resolve_subsume(b1, b2)
        self.events = [e for e in self.events if e[0] == "add"]

    def update(self, dt, R):
        for b in self.arr:
            if not b.exists:
                continue
            if not b.collided:
                b.vx += dt * b.fx / b.mass if b.mass != 0 else _div(dt * b.fx, b.mass)
                b.vy += dt * b.fy / b.mass if b.mass != 0 else _div(dt * b.fy, b.mass)
                b.vz += dt * b.fz / b.mass if b.mass != 0 else _div(dt * b.fz, b.mass)
            b.x += dt * b.vx
            b.y += dt * b.vy
            b.z += dt * b.vz
            b.collided = False
            b.r = R
            if math.isnan(b.x) or math.isnan(b.y) or math.isnan(b.z):
                b.exists = False

    def cycle_(self, R):
        arr = [b for b in self.arr if b.exists]
        for kind, b1, _ in reversed(self.events):
            if kind == "add":
                b1.r = R
                arr.append(b1)
        self.arr = arr
        self.events = []

    def step(self, dt, R):
        self.compute()
        self.process_mods()
        self.update(dt, R)
        self.cycle_(R)
        self.cycle += 1


def _div(a, b):
    """IEEE division by zero (Python raises where Go returns +-Inf/NaN)."""
    if a != a or a == 0:
        return math.nan
    return math.copysign(math.inf, a) * math.copysign(1.0, b)


def hexf(v):
    return float(v).hex()


def dump_state(sim):
    rows = []
    for b in sim.arr:
        flags = (1 if b.exists else 0) | (2 if b.is_sun else 0) | (4 if b.pinned else 0) | \
                (8 if b.telemetry else 0) | (16 if b.fragmenting else 0) | (32 if b.collided else 0)
        rows.append({"id": b.id, "collision": b.collision, "flags": flags, "frag_fragments": b.fr_fragments,
                     **{k: hexf(getattr(b, a)) for k, a in (
                         ("x", "x"), ("y", "y"), ("z", "z"), ("vx", "vx"), ("vy", "vy"), ("vz", "vz"),
                         ("radius", "radius"), ("mass", "mass"), ("frag_factor", "frag_factor"),
                         ("frag_step", "frag_step"), ("r", "r"), ("fx", "fx"), ("fy", "fy"), ("fz", "fz"),
                         ("frag_radius", "fr_radius"), ("frag_new_radius", "fr_new_radius"),
                         ("frag_mass", "fr_mass"), ("frag_cx", "fr_cx"), ("frag_cy", "fr_cy"),
                         ("frag_cz", "fr_cz"))}})
    return rows


def scenario(name, rows, dt, R, steps, seed=7, next_id=None):
    bodies = [Body(**r) for r in rows]
    inputs = dump_state(type("S", (), {"arr": bodies})())
    sim = Sim(bodies, seed, next_id if next_id is not None else len(rows))
    out = []
    for _ in range(steps):
        sim.step(dt, R)
        out.append({"state": dump_state(sim), "events": sim.handled, "next_id": sim.next_id})
    return {"name": name, "dt": dt, "R": R, "seed": seed, "next_id": next_id if next_id is not None else len(rows),
            "bodies": inputs, "steps": out}


def rnd_cluster(n, seed):
    s = seed
    vals = []

    def u():
        nonlocal s
        s = (s * 6364136223846793005 + 1442695040888963407) & MASK
        return (s >> 11) * 2.0 ** -53
    for i in range(n):
        vals.append(dict(id=i, x=u() * 20 - 10, y=u() * 20 - 10, z=u() * 20 - 10, vx=u() * 6 - 3, vy=u() * 6 - 3,
                         vz=u() * 6 - 3, mass=10 ** (8 + 4 * u()), radius=0.5 + 2.5 * u(),
                         collision=int(u() * 4) % 4, frag_factor=2 * u(), frag_step=400 * u()))
    return vals


SCENARIOS = [
    ("wp_compute_pair", [dict(id=1, x=1.0, y=1.0, z=1.0, mass=1.0, radius=1.0),
                         dict(id=2, x=22.0, y=22.0, z=22.0, mass=1.0, radius=1.0)], 1.0, 1.0, 3),
    ("simtest_three_body", [dict(id=0, x=20000.0, y=20000.0, z=20000.0, vx=-3.0, vy=-3.0, vz=-5.0, mass=1.0,
                                 radius=500.0, collision=SUBSUME, is_sun=True, pinned=True),
                            dict(id=1, mass=9e29, radius=60.0),
                            dict(id=2, x=-350.0, y=350.0, vx=530000000.0, vy=-500000000.0, mass=9e29, radius=60.0),
                            dict(id=3, x=350.0, y=350.0, vx=-530000000.0, vy=-500000000.0, mass=9e29, radius=60.0)],
     1e-7, 1.0, 12),
    ("head_on_elastic", [dict(id=0, x=-5.0, vx=3.0, mass=1e10, radius=1.0),
                         dict(id=1, x=5.0, vx=-3.0, mass=2e10, radius=1.5)], 0.5, 1.0, 6),
    ("subsume_triple", [dict(id=0, mass=1e9, radius=5.0, collision=SUBSUME),
                        dict(id=1, x=0.5, mass=1e3, radius=0.2, collision=SUBSUME),
                        dict(id=2, x=1.0, mass=2e9, radius=4.0, collision=SUBSUME),
                        dict(id=3, x=50.0, mass=1e3, radius=0.2, collision=SUBSUME)], 0.01, 1.0, 3),
    ("fragment_impact", [dict(id=0, x=-2.0, vx=40.0, vy=1.0, mass=1e6, radius=1.0),
                         dict(id=1, x=0.5, vx=-5.0, vy=0.3, vz=0.2, mass=5e6, radius=2.0, collision=FRAGMENT,
                              frag_factor=0.1, frag_step=2.0)], 0.01, 1.0, 4),
    ("restitution_cluster", rnd_cluster(12, 99), 0.05, 0.8, 8),
]


def main():
    for name, rows, dt, R, steps in SCENARIOS:
        fx = scenario(name, rows, dt, R, steps)
        with open(os.path.join(HERE, name + ".json"), "w") as fh:
            json.dump(fx, fh, indent=0, separators=(",", ":"))
        print(name, "bodies after:", len(fx["steps"][-1]["state"]), "events:",
              sum(len(s["events"]) for s in fx["steps"]))


if __name__ == "__main__":
    main()

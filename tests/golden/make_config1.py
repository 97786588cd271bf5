"""The 256-body adaptive RKF78 configuration at its full length as a scenario
file, and the reference program's run of it.

Writes tests/golden/scenarios/config1_1000yr.xml from the seeded generator
(solaris_gb300.scenarios.config1: 1 star, giants of 1e-3 and 3e-4 Msun at 5.2
and 9.5 AU, 253 test particles with a ~ U(3, 12) AU; phases in AU and AU/day
written with round-trip precision, so the file reproduces the generator's
state bit for bit), then runs the reference's own Solaris program on it
(oracle/_ref/solaris_counted: the program built from the reference sources by
oracle/Makefile, with counters of its driver calls and force evaluations
wrapped around its unchanged objects) and
keeps in tests/golden/scenarios/config1_1000yr/:
  Integrals.dat, TwoBodyAffair.dat   the reference's output files;
  summary.json                       the accepted and rejected step counts
                                     (from the wrapped counters), the
                                     event list, the energy drift and the
                                     program's wall time on this machine.
The phases file (14 MB for 1,000 years) is not kept.

    python tests/golden/make_config1.py [reference source root]
"""
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SCENARIOS = os.path.join(HERE, "scenarios")
NAME = "config1_1000yr"

# Events the run watches: the ejection sphere and the hit-centrum radius
# (AU), and the collision factor; chosen so that the giants scatter some
# test particles across one of them within 1,000 years.
EJECTION_AU = 15.0
HIT_CENTRUM_AU = 1.0
OUTPUT_YEARS = 100.0


def write_xml(path):
    sys.path.insert(0, ROOT)
    from solaris_gb300 import abi, scenarios
    s = scenarios.config1()
    y = s.y0.reshape(-1, 6)
    lines = ['<?xml version="1.0" encoding="utf-8"?>',
             '<Simulation name="config1_1000yr" description="1 star, giants of 1e-3 and 3e-4 Msun at 5.2 and 9.5 AU, '
             '253 test particles (a ~ U(3, 12) AU); adaptive RKF78, epsilon 1e-10, 1000 years.">',
             '  <Settings enableDistinctStartTimes="false" barycentric="false">',
             '    <Output>', '      <Phases>Phases.dat</Phases>', '      <Integrals>Integrals.dat</Integrals>',
             '      <TwoBodyAffair>TwoBodyAffair.dat</TwoBodyAffair>', '    </Output>',
             '    <Integrator xmlns:xsi="http://www.w3.org/2001/XMLSchema-instance" '
             'xmlns:xsd="http://www.w3.org/2001/XMLSchema" xsi:type="RungeKutta78">',
             '      <Accuracy value="-10" />', '    </Integrator>',
             f'    <TimeLine length="1000" output="{OUTPUT_YEARS:g}" unit="year" />',
             f'    <Ejection value="{EJECTION_AU:g}" unit="au" />',
             f'    <HitCentrum value="{HIT_CENTRUM_AU:g}" unit="au" />',
             '  </Settings>', '  <BodyGroupList>', '    <BodyGroup description="star, giants and test particles">',
             '      <Items>',
             '        <Body type="centralbody" name="Star" guid="00000000-0000-0000-0000-000000000001">',
             '          <Characteristics>', '            <Mass value="1" unit="solar" />',
             '            <Radius value="1" unit="solarradius" />', '          </Characteristics>', '        </Body>']
    for i in range(1, s.n):
        giant = s.type[i] == abi.GIANT_PLANET
        kind = "giantplanet" if giant else "testparticle"
        guid = f"00000000-0000-0000-0000-{i + 1:012d}"
        lines.append(f'        <Body type="{kind}" name="B{i}" guid="{guid}">')
        lines.append('          <Phase>')
        lines.append(f'            <Position x="{float(y[i, 0])!r}" y="{float(y[i, 1])!r}" z="{float(y[i, 2])!r}" unit="au" />')
        lines.append(f'            <Velocity x="{float(y[i, 3])!r}" y="{float(y[i, 4])!r}" z="{float(y[i, 5])!r}" unit="auday" />')
        lines.append('          </Phase>')
        if giant:
            lines += ['          <Characteristics>', f'            <Mass value="{float(s.mass[i])!r}" unit="solar" />',
                      '            <Density value="1.33" unit="gcm3" />', '          </Characteristics>']
        lines.append('        </Body>')
    lines += ['      </Items>', '    </BodyGroup>', '  </BodyGroupList>', '</Simulation>', '']
    with open(path, "w") as f:
        f.write("\n".join(lines))


def counters(stderr):
    """Accepted steps (driver calls) and rejected attempts of the reference
    program, from the counters oracle/ref_counters.cpp wraps around it: an
    accepted RKF78 driver call evaluates 13 times, a rejected attempt 12."""
    m = re.search(r"ref_counters: driver_calls (\d+) force_evaluations (\d+)", stderr)
    if not m:
        raise SystemExit("no counters in the reference program's output")
    calls, evals = int(m.group(1)), int(m.group(2))
    rejected, rest = divmod(evals - 13 * calls, 12)
    if rest:
        raise SystemExit(f"{evals} evaluations are not 13 x {calls} + 12 x rejected")
    return dict(accepted=calls, rejected=rejected, evaluations=evals)


def run(ref_root=None):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.dirname(HERE))
    import oracle
    ref_root = ref_root or oracle.REFERENCE_SRC
    from scenario_files import read_affairs, read_integrals
    xml = os.path.join(SCENARIOS, NAME + ".xml")
    write_xml(xml)
    if not oracle.build_reference(ref_root):
        raise SystemExit("the reference sources are not available")
    prog = os.path.join(oracle.REF_DIR, "solaris_counted")
    out = os.path.join(SCENARIOS, NAME)
    with tempfile.TemporaryDirectory() as tmp:
        shutil.copy(xml, tmp)
        t0 = time.perf_counter()
        r = subprocess.run([prog, "-i", os.path.join(tmp, NAME + ".xml")], cwd=tmp, capture_output=True, text=True,
                           env=dict(os.environ, OSTYPE="linux"), timeout=3600)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            raise SystemExit(f"the reference program failed\n{r.stdout}\n{r.stderr}")
        shutil.rmtree(out, ignore_errors=True)
        os.makedirs(out)
        for f in ("Integrals.dat", "TwoBodyAffair.dat"):
            if os.path.exists(os.path.join(tmp, f)):
                shutil.copy(os.path.join(tmp, f), out)
            else:
                open(os.path.join(out, f), "wb").close()
    _, integ = read_integrals(os.path.join(out, "Integrals.dat"))
    affairs = read_affairs(os.path.join(out, "TwoBodyAffair.dat"))
    e0, e1 = integ[0][1][15], integ[-1][1][15]
    summary = dict(counters(r.stderr), wall_s=wall, machine=os.uname().machine, stdout=r.stdout[-2000:],
                   events=[dict(type=a["type"], id1=a["id1"], id2=a["id2"], time=a["time"]) for a in affairs],
                   energy_first=e0, energy_last=e1, energy_rel_drift=abs((e1 - e0) / e0),
                   records=len(integ), final_time=integ[-1][0])
    with open(os.path.join(out, "summary.json"), "w") as f:
        json.dump(summary, f, indent=1)
    print(json.dumps({k: v for k, v in summary.items() if k not in ("stdout",)}, indent=1))


if __name__ == "__main__":
    run(*sys.argv[1:])

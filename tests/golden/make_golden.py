"""Writes tests/golden/kat_check.json: known-answer cases for the report rule.

Each case restates one of the reference's own GPU tests at the level of the
check pass (clauses, per-slot assignments, expected reports), with the
expected reports taken from that test's assertions - not computed by the
oracle - so the fixture pins the oracle as well as the CUDA path. Paths are
relative to the GpuShareSat repository.

Values: 'T' true, 'F' false, 'U' undefined; lit = 2*var + sign.
Expected reports are (clause index, word, slot) triples; word = solver here.
"""
import json
import os


def lit(v, neg=False):
    return 2 * v + (1 if neg else 0)


def case_find_clauses_multithread():
    # glucose-syrup/test/GpuSolverTest.cu:394-454 - one solver, one assignment
    # x0=F x1=T x2=U; clauses (x0|x1), (x0|~x1), (~x1|x2). The test pops exactly
    # (x0|~x1) (all false) and (~x1|x2) (one undefined), and nothing else.
    return {
        "name": "find_clauses_multithread",
        "source": "glucose-syrup/test/GpuSolverTest.cu:394-454",
        "n_vars": 3,
        "clauses": [[lit(0), lit(1)], [lit(0), lit(1, True)], [lit(1, True), lit(2)]],
        "words": [{"solver": 0, "slots": ["FTU"]}],
        "expected": [[1, 0, 0], [2, 0, 0]],
    }


def case_clauses_assigs_reported():
    # glucose-syrup/test/GpuSolverTest.cu:343-391 - unit clauses x0, x1, x2;
    # solver 0 sends (F,T,T) then (T,F,F); solver 1 sends (T,F,T); solver 2
    # sends nothing. The test expects 3, 1 and 0 imported clauses: solver 0's
    # first assignment reports x0, its second x1 and x2; solver 1's reports x1.
    return {
        "name": "clauses_assigs_reported_pass1",
        "source": "glucose-syrup/test/GpuSolverTest.cu:343-381",
        "n_vars": 3,
        "clauses": [[lit(0)], [lit(1)], [lit(2)]],
        "words": [{"solver": 0, "slots": ["FTT", "TFF"]},
                  {"solver": 1, "slots": ["TFT"]},
                  {"solver": 2, "slots": []}],
        "expected": [[0, 0, 0], [1, 0, 1], [1, 1, 0], [2, 0, 1]],
    }


def case_clauses_assigs_reported_pass2():
    # glucose-syrup/test/GpuSolverTest.cu:383-390 - solver 0 then sets x1=T and
    # sends again (x0=T x1=T x2=F, its third assignment, slot 2 of its ring);
    # the test expects exactly one clause (x2) for solver 0 and none for solver 1.
    return {
        "name": "clauses_assigs_reported_pass2",
        "source": "glucose-syrup/test/GpuSolverTest.cu:383-390",
        "n_vars": 3,
        "clauses": [[lit(0)], [lit(1)], [lit(2)]],
        "words": [{"solver": 0, "slots": [None, None, "TTF"]},
                  {"solver": 1, "slots": []}],
        "expected": [[2, 0, 2]],
    }


def case_one_assignment_then_two():
    # glucose-syrup/test/GpuSolverTest.cu:486-508 - clause (~x0|~x1|x2). First
    # pass: trail x0 -> nothing. Second pass: trail x0,x3 then x0,x3,x1 (two
    # assignments); exactly one report, for the second of them.
    return {
        "name": "one_assignment_then_two_pass2",
        "source": "glucose-syrup/test/GpuSolverTest.cu:486-508",
        "n_vars": 4,
        "clauses": [[lit(0, True), lit(1, True), lit(2)]],
        "words": [{"solver": 0, "slots": [None, "TUUT", "TTUT"]}],
        "expected": [[0, 0, 2]],
    }


def case_many_units_all_at_once():
    # glucose-syrup/test/GpuSolverTest.cu:696-724 - 4000 unit clauses x_i; the
    # solver's one assignment sets x_i true for i % 3 == 0. Every other unit
    # (variable undefined) reports: 4000 - ceil(4000/3) = 2666 clauses.
    n = 4000
    slot = "".join("T" if i % 3 == 0 else "U" for i in range(n))
    return {
        "name": "many_units_all_at_once",
        "source": "glucose-syrup/test/GpuSolverTest.cu:696-724",
        "n_vars": n,
        "clauses": [[lit(i)] for i in range(n)],
        "words": [{"solver": 0, "slots": [slot]}],
        "expected": [[i, 0, 0] for i in range(n) if i % 3 != 0],
    }


def case_solver_passes_many_assignments():
    # glucose-syrup/test/GpuSolverTest.cu:949-981 - 32 clauses (~x_{2i}|x_{2i+1});
    # assignment i sets only x_{2i} true. 32 assignments in one pass, 32 imports:
    # clause i reports exactly for assignment i (slot i).
    n_vars = 64
    slots = []
    for i in range(32):
        s = ["U"] * n_vars
        s[2 * i] = "T"
        slots.append("".join(s))
    return {
        "name": "solver_passes_many_assignments",
        "source": "glucose-syrup/test/GpuSolverTest.cu:949-981",
        "n_vars": n_vars,
        "clauses": [[lit(2 * i, True), lit(2 * i + 1)] for i in range(32)],
        "words": [{"solver": 0, "slots": slots}],
        "expected": [[i, 0, i] for i in range(32)],
    }


def case_true_literal_blocks():
    # glucose-syrup/test/GpuSolverTest.cu:394-454 (clause x0|x1 under x1=T) and
    # README.md:6-12: a true literal means the clause is satisfied, so it never
    # reports, even when every other literal is false.
    return {
        "name": "true_literal_blocks",
        "source": "glucose-syrup/test/GpuSolverTest.cu:394-454; README.md:6-12",
        "n_vars": 4,
        "clauses": [[lit(0), lit(1), lit(2)], [lit(3)], [lit(3, True)]],
        "words": [{"solver": 0, "slots": ["FTFT", "FFUT", "FUUF"]}],
        # slot0: c0 has x1 true -> no; c1 x3 true -> no; c2 ~x3 false -> all false -> yes
        # slot1: c0 F,F,U -> one undef -> yes; c1 x3=T no; c2 yes
        # slot2: c0 F,U,U -> two undef -> no; c1 x3=F -> yes; c2 ~x3 true -> no
        "expected": [[0, 0, 1], [1, 0, 2], [2, 0, 0], [2, 0, 1]],
    }


CASES = [
    case_find_clauses_multithread(),
    case_clauses_assigs_reported(),
    case_clauses_assigs_reported_pass2(),
    case_one_assignment_then_two(),
    case_many_units_all_at_once(),
    case_solver_passes_many_assignments(),
    case_true_literal_blocks(),
]


def main():
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat_check.json")
    with open(out, "w") as f:
        json.dump({"generated_by": "tests/golden/make_golden.py", "cases": CASES}, f, indent=0)
    print(out)


if __name__ == "__main__":
    main()

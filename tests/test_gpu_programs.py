"""Hybrid programs (Quil instruction set) on the GPU engine: the behaviour the
reference's own program tests check (tests/test_programs.py of the
reference: labels, jumps, halts, waits, reset, measurement, Bell and QAOA
programs), seeded Call programs against states computed by the reference's
Program.run (tests/golden/programs.npz), and the measurement reduction
against the oracle."""
import numpy as np
import pytest

from oracle import qf_oracle as orc

pytestmark = pytest.mark.gpu


def test_empty_and_nop():
    import quantumflow_gb300 as qf
    ket = qf.Program().run()
    assert ket.qubits == () and ket.qubit_nb == 0
    prog = qf.Program()
    prog += qf.Nop()
    prog.run()
    assert qf.Nop().qubits == () and qf.Nop().qubit_nb == 0


def test_labels_and_jumps():
    import quantumflow_gb300 as qf
    from quantumflow_gb300.programs import TARGETS, PC
    prog = qf.Program()
    prog += qf.Label("Here")
    prog += qf.Nop()
    prog += qf.Label("There")
    assert prog.run().memory[TARGETS] == {"Here": 0, "There": 2}

    ro = qf.Register()
    prog = qf.Program()
    prog += qf.Move(ro[0], 0)
    prog += qf.Jump("There")
    prog += qf.Not(ro[0])
    prog += qf.Label("There")
    prog += qf.Not(ro[0])
    assert prog.run().memory[ro[0]] == 1
    prog += qf.JumpWhen("There", ro[0])
    assert prog.run().memory[ro[0]] == 0
    prog += qf.Not(ro[0])
    prog += qf.JumpUnless("There", ro[0])
    assert prog.run().memory[ro[0]] == 1

    prog = qf.Program()
    prog += qf.Move(ro[0], 0)
    prog += qf.Halt()
    prog += qf.Not(ro[0])
    ket = prog.run()
    assert ket.memory[PC] == -1 and ket.memory[ro[0]] == 0

    prog = qf.Program()
    prog += qf.Move(ro[0], 0)
    for _ in range(3):
        prog += qf.Wait()
        prog += qf.Not(ro[0])
    assert prog.run().memory[ro[0]] == 1


def test_classical_operations():
    import quantumflow_gb300 as qf
    a, b = qf.Register("a", "INT"), qf.Register("b", "REAL")
    prog = qf.Program()
    prog += qf.Declare("a", "INT", 3)
    prog += qf.Move(a[0], 7)
    prog += qf.Move(a[1], 3)
    prog += qf.Add(a[0], a[1])        # 10
    prog += qf.Mul(a[0], 2)           # 20
    prog += qf.Sub(a[0], a[1])        # 17
    prog += qf.Move(b[0], 1.0)
    prog += qf.Div(b[0], 4)           # 0.25
    prog += qf.Exchange(a[1], a[2])   # a1 = 0, a2 = 3
    prog += qf.Neg(a[2])              # -3
    prog += qf.Xor(a[1], 1)
    prog += qf.GT(a[2], a[0], a[1])   # 17 > 1
    prog += qf.EQ(b[1], a[1], a[1])
    ket = prog.run()
    m = ket.memory
    assert m[a[0]] == 17 and m[a[1]] == 1 and m[a[2]] == 1 and m[b[0]] == 0.25 and m[b[1]]
    assert str(prog[0]) == "DECLARE a INT [3]"


def test_reset_and_measure():
    import quantumflow_gb300 as qf
    ro = qf.Register()
    prog = qf.Program()
    prog += qf.Move(ro[0], 1)
    prog += qf.Call("X", params=[], qubits=[0])
    prog += qf.Reset()
    prog += qf.Measure(0, ro[1])
    ket = prog.run()
    assert ket.qubits == (0,) and ket.memory[ro[0]] == 1 and ket.memory[ro[1]] == 0

    prog = qf.Program()
    prog += qf.Call("X", params=[], qubits=[0])
    prog += qf.Call("X", params=[], qubits=[1])
    prog += qf.Reset(0)
    prog += qf.Measure(0, ("b", 0))
    prog += qf.Measure(1, ("b", 1))
    ket = prog.run()
    assert ket.memory[("b", 0)] == 0 and ket.memory[("b", 1)] == 1


def test_measure_until_and_bell_statistics():
    import quantumflow_gb300 as qf
    np.random.seed(3)
    prog = qf.Program()
    prog += qf.Move(("c", 2), 1)
    prog += qf.Label("redo")
    prog += qf.Call("X", [], [0])
    prog += qf.Call("H", [], [0])
    prog += qf.Measure(0, ("c", 2))
    prog += qf.JumpUnless("redo", ("c", 2))
    assert prog.run().memory[("c", 2)] == 1

    ro = qf.Register()
    bell = qf.Program()
    bell += qf.Call("H", [], [0])
    bell += qf.Call("CNOT", [], [0, 1])
    assert qf.states_close(bell.run(), qf.ghz_state(2))
    bell += qf.Measure(0, ro[0])
    bell += qf.Measure(1, ro[1])
    ones = 0
    for _ in range(200):
        m = bell.run().memory
        assert m[ro[0]] == m[ro[1]]
        ones += m[ro[0]]
    assert 60 < ones < 140  # binomial(200, 1/2): 5 sigma


def test_occupation_basis_and_qaoa_program(golden):
    import quantumflow_gb300 as qf
    prog = qf.Program()
    prog += qf.Call("X", [], [0])
    prog += qf.Call("X", [], [1])
    prog += qf.Call("I", [], [2])
    prog += qf.Call("I", [], [3])
    ket = prog.run()
    assert ket.qubits == (0, 1, 2, 3)
    probs = qf.asarray(ket.probabilities())
    assert probs[1, 1, 0, 0] == 1.0 and probs[1, 1, 0, 1] == 0.0

    prog = qf.Program()
    prog += qf.Call("RY", [np.pi / 2], [0])
    prog += qf.Call("RX", [np.pi], [0])
    prog += qf.Call("RY", [np.pi / 2], [1])
    prog += qf.Call("RX", [np.pi], [1])
    prog += qf.Call("CNOT", [], [0, 1])
    prog += qf.Call("RX", [-np.pi / 2], [1])
    prog += qf.Call("RY", [4.71572463191], [1])
    prog += qf.Call("RX", [np.pi / 2], [1])
    prog += qf.Call("CNOT", [], [0, 1])
    prog += qf.Call("RX", [-2 * 2.74973750579], [0])
    prog += qf.Call("RX", [-2 * 2.74973750579], [1])
    assert qf.states_close(prog.run(), qf.State(golden["programs"]["wf_true"].reshape(2, 2)))


def test_exceptions_and_text():
    import quantumflow_gb300 as qf
    prog = qf.Program()
    prog += qf.Call("NOT_A_GATE", [], [0])
    with pytest.raises(RuntimeError):
        prog.run()
    prog = qf.Program()
    prog += qf.Call("BELL", params=[], qubits=[])
    assert str(prog) == "BELL\n"
    circ = qf.DefCircuit("CIRCX", {})
    circ += qf.Call("X", params=[], qubits=[0])
    prog = qf.Program()
    prog += circ
    prog += qf.Call("CIRCX", params=[], qubits=[0])
    assert str(prog) == "DEFCIRCUIT CIRCX:\n    X 0\n\nCIRCX 0\n"
    assert prog.qubits == [0]
    assert qf.Include("somefile.quil", qf.Program()).quil() == 'INCLUDE "somefile.quil"'


@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 2e-5)])
def test_seeded_call_programs_vs_reference(golden, dtype, tol):
    """Programs of 40..200 named-gate calls: one fused launch per run of
    calls, equal to the reference's Program.run state."""
    import quantumflow_gb300 as qf
    g = golden["programs"]
    for case in range(3):
        nq = int(g[f"p{case}_nq"])
        prog = qf.Program()
        for name, ps, qs in zip(g[f"p{case}_names"], g[f"p{case}_params"], g[f"p{case}_qubits"]):
            prog += qf.Call(str(name), [float(p) for p in ps if not np.isnan(p)], [int(q) for q in qs if q >= 0])
        ket = prog.run(qf.zero_state(nq, dtype=dtype))
        assert np.max(np.abs(ket.asarray().reshape(-1) - g[f"p{case}_state"])) < tol


@pytest.mark.parametrize("n", [1, 6, 17])
def test_qubit_probabilities_vs_oracle(n):
    import quantumflow_gb300 as qf
    from quantumflow_gb300.states import _reduce
    rng = np.random.default_rng(n)
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    v /= np.linalg.norm(v)
    ket = qf.State(v.reshape([2] * n))
    probs = orc.probabilities(v.reshape([2] * n))
    for axis in sorted({0, n // 2, n - 1}):
        p0, p1 = _reduce("qf_qubit_probabilities", ket.buffer.compute(), nout=2, extra=(axis,))
        ref0 = float(np.take(probs, 0, axis=axis).sum())
        assert abs(p0 - ref0) < 1e-13 and abs(p0 + p1 - 1) < 1e-13


def test_measure_collapses_like_projection():
    """Measure leaves exactly the normalised projection for the outcome it
    reports (quantumflow/stdops.py:53-64)."""
    import quantumflow_gb300 as qf
    n = 9
    rng = np.random.default_rng(11)
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    v /= np.linalg.norm(v)
    np.random.seed(5)
    for q in (0, 4, 8):
        ket = qf.State(v.reshape([2] * n)).update({"m": -1})
        out = qf.Measure(q, "m").run(ket)
        bit = out.memory["m"]
        ref = v.reshape([2] * n).copy()
        sl = [slice(None)] * n
        sl[q] = 1 - bit
        ref[tuple(sl)] = 0
        ref /= np.linalg.norm(ref)
        assert np.max(np.abs(out.asarray() - ref)) < 1e-12

"""Initiator rules (src/DictVectors/initiators.jl:132-234).  A rule is a property of the walker
vector (InitiatorDVec(...; initiator), or ProjectorMonteCarloProblem(...; initiator)); the step
kernels classify every contribution by its parent (initiators.jl:142-157) and combine the
per-class sums by the rule."""


class InitiatorRule:
    code = 0

    def __init__(self, threshold=1.0):
        self.threshold = float(threshold)

    def __eq__(self, other):
        return type(self) is type(other) and self.threshold == other.threshold

    def __repr__(self):
        return f"{type(self).__name__}({self.threshold})"


class NonInitiator(InitiatorRule):
    """NonInitiator() (initiators.jl:227-236): no initiator approximation."""
    code = 0

    def __init__(self):
        super().__init__(1.0)

    def __repr__(self):
        return "NonInitiator()"


class Initiator(InitiatorRule):
    """Initiator(threshold=1) (initiators.jl:132-140): initiators spawn anywhere, non-initiators
    only onto initiators."""
    code = 1


class SimpleInitiator(InitiatorRule):
    """SimpleInitiator(threshold=1) (initiators.jl:175-183): non-initiators do not spawn."""
    code = 2


class CoherentInitiator(InitiatorRule):
    """CoherentInitiator(threshold=1) (initiators.jl:202-214): non-initiator spawns also
    survive on a non-initiator when together they exceed the threshold."""
    code = 3


def initiator_rule(x) -> InitiatorRule:
    """`initiator = true / false / rule` of ProjectorMonteCarloProblem
    (projector_monte_carlo_problem.jl:221-223)."""
    if x is True:
        return Initiator()
    if x is False or x is None:
        return NonInitiator()
    if not isinstance(x, InitiatorRule):
        raise ValueError("initiator must be true, false or an InitiatorRule")
    return x

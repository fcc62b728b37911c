"""The five MC moves (chromo/mc/move_funcs.pyx).

Proposals are generated inside the GPU kernel, so these objects identify a
move kind to ``MCAdapter`` / the controllers; their ``__name__`` is the
reference function name.  Calling one directly is not supported: it would
need the reference's per-polymer trial arrays, which this implementation
does not keep on the host.
"""


class MoveFunction:
    def __init__(self, name, kind):
        self.__name__ = name
        self.kind = kind

    def __call__(self, polymer=None, amp_move=None, amp_bead=None):
        raise NotImplementedError(
            f"{self.__name__} proposals run inside the GPU kernel; use chromo_gb300.mc.mc_sim")

    def __repr__(self):
        return f"<move {self.__name__}>"


crank_shaft = MoveFunction("crank_shaft", 0)
end_pivot = MoveFunction("end_pivot", 1)
slide = MoveFunction("slide", 2)
tangent_rotation = MoveFunction("tangent_rotation", 3)
change_binding_state = MoveFunction("change_binding_state", 4)
move_list = [crank_shaft, end_pivot, slide, tangent_rotation, change_binding_state]

"""Acceptance tracking (chromo/util/mc_stat.py:45-208).

The exponentially weighted moving average acceptance rate,
acc <- alpha * accepted + (1 - alpha) * acc with alpha = 2 / (n + 1), is
updated on the GPU after every move; after ``mc_sim`` returns it is copied
back into ``acceptance_rate``.  Per-move logs are not recorded on the GPU path
(the reference's hot loop runs with ``log_move = False``,
chromo/mc/mc_sim.pyx:173-180).
"""


class AcceptanceTracker:
    def __init__(self, log_dir: str, log_file_prefix: str, moves_in_average: float):
        self.log_dir = log_dir
        self.log_file_prefix = log_file_prefix
        self.alpha = 2 / (moves_in_average + 1)
        self.acceptance_rate = 0

    def update_acceptance_rate(self, accept: float, log_update: int = 0):
        self.acceptance_rate = (self.alpha * accept) + (1 - self.alpha) * self.acceptance_rate

    def create_log_file(self, snapshot=0):
        pass

    def save_move_log(self, snapshot=0):
        pass

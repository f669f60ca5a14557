"""Life-like rule helpers (reference ``xentica/tools/rules.py:5-37``).

Rule integers hold birth counts in bits 0-8 and survival counts in bits 9-17.
"""
import re


class LifeLike:
    """Conversions between Golly notation and rule integers."""

    @staticmethod
    def golly2int(golly_str):
        """``"B3/S23"`` -> ``6152``."""
        born, sustained = re.sub("[^0-9/]", "", golly_str).split("/", 1)
        return sum(1 << (int(i) + 9) for i in sustained) + sum(1 << int(i) for i in born)

    @staticmethod
    def int2golly(rule):
        """``6152`` -> ``"B3/S23"``."""
        sustained = (rule >> 9) & 0b111111111
        born = rule & 0b111111111
        sus = ''.join(str(i) * ((sustained >> i) & 1) for i in range(9))
        bor = ''.join(str(i) * ((born >> i) & 1) for i in range(9))
        return "B%s/S%s" % (bor, sus)

"""Number formatting (reference ``xentica/utils/formatters.py:4-26``)."""


def sizeof_fmt(num, suffix=''):
    """Humanise ``num`` by powers of 1000, e.g. ``11234`` -> ``"11.23K"``."""
    if abs(num) < 1000:
        return "%s%s" % (num, suffix)
    for unit in ['K', 'M', 'G', 'T', 'P', 'E', 'Z']:
        num /= 1000.0
        if abs(num) < 1000.0:
            return "%.2f%s%s" % (num, unit, suffix)
    num /= 1000.0
    return "%.2f%s%s" % (num, 'Y', suffix)

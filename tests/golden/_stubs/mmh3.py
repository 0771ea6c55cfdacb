"""Empty stand-in so lettuce imports in a container without this optional
dependency; it is not on lettuce's arithmetic path (file output / module naming only)."""
def hash(*a, **k):
    return 0

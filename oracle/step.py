"""Oracle step driver (filled in below)."""
__all__ = []

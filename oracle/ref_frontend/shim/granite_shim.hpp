// TEST INFRASTRUCTURE ONLY.  Stand-ins for the Granite utility types the
// reference's CPU frontend uses (Util::IntrusivePtr, the intrusive hash maps,
// ObjectPool, DynamicArray, Hasher, bit helpers, logging).  Granite itself is
// an empty submodule in the reference, so these are written here from the
// behaviour the frontend relies on: reference-counted handles, hash-keyed maps
// that own or borrow their entries, and an FNV-style hasher (hash values are
// only compared for equality).
#pragma once
#include <assert.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <memory>
#include <unordered_map>
#include <utility>
#include <vector>

#ifndef LOGE
#define LOGE(...) fprintf(stderr, __VA_ARGS__)
#endif
#ifndef LOGW
#define LOGW(...) ((void)0)
#endif
#ifndef LOGI
#define LOGI(...) ((void)0)
#endif

namespace Util
{
using Hash = uint64_t;

class Hasher
{
public:
	void u32(uint32_t v) { h = (h * 0x100000001b3ull) ^ v; }
	void s32(int32_t v) { u32(uint32_t(v)); }
	void u64(uint64_t v) { u32(uint32_t(v)); u32(uint32_t(v >> 32)); }
	void f32(float f) { uint32_t u; memcpy(&u, &f, 4); u32(u); }
	void data(const void *p, size_t n)
	{
		const uint8_t *b = static_cast<const uint8_t *>(p);
		for (size_t i = 0; i < n; i++)
			u32(b[i]);
	}
	Hash get() const { return h; }

private:
	Hash h = 0xcbf29ce484222325ull;
};

inline uint32_t leading_zeroes(uint32_t v) { return v ? uint32_t(__builtin_clz(v)) : 32u; }
inline uint32_t trailing_zeroes(uint32_t v) { return v ? uint32_t(__builtin_ctz(v)) : 32u; }
inline uint32_t leading_zeroes64(uint64_t v) { return v ? uint32_t(__builtin_clzll(v)) : 64u; }
inline uint32_t trailing_zeroes64(uint64_t v) { return v ? uint32_t(__builtin_ctzll(v)) : 64u; }

template <typename T>
inline void for_each_bit(uint32_t value, const T &func)
{
	while (value)
	{
		uint32_t bit = trailing_zeroes(value);
		func(bit);
		value &= value - 1u;
	}
}

template <typename T>
inline void for_each_bit64(uint64_t value, const T &func)
{
	while (value)
	{
		uint32_t bit = trailing_zeroes64(value);
		func(bit);
		value &= value - 1u;
	}
}

struct SingleThreadCounter
{
};

template <typename T, typename Deleter = std::default_delete<T>, typename Counter = SingleThreadCounter>
class IntrusivePtrEnabled
{
public:
	void add_reference() { refs++; }
	void release_reference()
	{
		if (--refs == 0)
			Deleter()(static_cast<T *>(this));
	}

private:
	size_t refs = 1;
};

template <typename T>
class IntrusivePtr
{
public:
	IntrusivePtr() = default;
	explicit IntrusivePtr(T *handle) : p(handle) {}
	IntrusivePtr(const IntrusivePtr &o) : p(o.p) { if (p) p->add_reference(); }
	IntrusivePtr(IntrusivePtr &&o) noexcept : p(o.p) { o.p = nullptr; }
	~IntrusivePtr() { reset(); }
	IntrusivePtr &operator=(const IntrusivePtr &o)
	{
		if (this != &o)
		{
			if (o.p)
				o.p->add_reference();
			reset();
			p = o.p;
		}
		return *this;
	}
	IntrusivePtr &operator=(IntrusivePtr &&o) noexcept
	{
		if (this != &o)
		{
			reset();
			p = o.p;
			o.p = nullptr;
		}
		return *this;
	}
	void reset()
	{
		if (p)
			p->release_reference();
		p = nullptr;
	}
	T *get() const { return p; }
	T *operator->() const { return p; }
	T &operator*() const { return *p; }
	explicit operator bool() const { return p != nullptr; }
	bool operator==(const IntrusivePtr &o) const { return p == o.p; }
	bool operator!=(const IntrusivePtr &o) const { return p != o.p; }

private:
	T *p = nullptr;
};

template <typename T>
class IntrusiveHashMapEnabled
{
public:
	Hash get_hash() const { return intrusive_hash; }
	void set_hash(Hash h) { intrusive_hash = h; }

private:
	Hash intrusive_hash = 0;
};

template <typename T>
struct IntrusivePODWrapper : IntrusiveHashMapEnabled<IntrusivePODWrapper<T>>
{
	template <typename U>
	explicit IntrusivePODWrapper(U &&v) : value(std::forward<U>(v)) {}
	T &get() { return value; }
	const T &get() const { return value; }
	T value = {};
};

// Borrowing map: entries are owned elsewhere.
template <typename T>
class IntrusiveHashMapHolder
{
public:
	T *find(Hash h) const
	{
		auto it = map.find(h);
		return it == map.end() ? nullptr : it->second;
	}
	// Inserts value unless its hash is present.  Returns nullptr when it was
	// inserted; otherwise value is set to the present entry and the caller's
	// object is returned for it to dispose of.
	T *insert_yield(T *&value)
	{
		auto it = map.find(value->get_hash());
		if (it != map.end())
		{
			T *mine = value;
			value = it->second;
			return mine;
		}
		map.emplace(value->get_hash(), value);
		return nullptr;
	}
	T *insert_replace(T *value)
	{
		T *old = find(value->get_hash());
		map[value->get_hash()] = value;
		return old;
	}
	void erase(T *value)
	{
		auto it = map.find(value->get_hash());
		if (it != map.end() && it->second == value)
			map.erase(it);
	}
	void clear() { map.clear(); }

private:
	std::unordered_map<Hash, T *> map;
};

// Owning map.
template <typename T>
class IntrusiveHashMap
{
public:
	T *find(Hash h) const
	{
		auto it = map.find(h);
		return it == map.end() ? nullptr : it->second.get();
	}
	template <typename... P>
	T *emplace_replace(Hash h, P &&...p)
	{
		std::unique_ptr<T> v(new T(std::forward<P>(p)...));
		v->set_hash(h);
		T *raw = v.get();
		map[h] = std::move(v);
		return raw;
	}
	template <typename... P>
	T *emplace_yield(Hash h, P &&...p)
	{
		if (T *t = find(h))
			return t;
		return emplace_replace(h, std::forward<P>(p)...);
	}
	void erase(Hash h) { map.erase(h); }
	void clear() { map.clear(); }

private:
	std::unordered_map<Hash, std::unique_ptr<T>> map;
};

template <typename T>
class ObjectPool
{
public:
	template <typename... P>
	T *allocate(P &&...p) { return new T(std::forward<P>(p)...); }
	void free(T *p) { delete p; }
};

template <typename T>
class DynamicArray
{
public:
	void reserve(size_t n)
	{
		if (n > v.size())
			v.resize(n);
	}
	T *data() { return v.data(); }
	const T *data() const { return v.data(); }
	size_t size() const { return v.size(); }

private:
	std::vector<T> v;
};

// Removes the elements pred selects by moving the last kept elements into
// their slots (order is not kept); returns the new end.
template <typename Iter, typename Pred>
Iter unstable_remove_if(Iter first, Iter last, Pred &&pred)
{
	while (first != last)
	{
		if (pred(*first))
		{
			--last;
			if (first != last)
				std::swap(*first, *last);
		}
		else
			++first;
	}
	return last;
}
}
